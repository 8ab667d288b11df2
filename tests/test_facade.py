"""The C++ IrradianceProbes class (include/irradiance_probes.hpp) over the C
ABI: a compiled host program (tests/native/irradiance_probes_facade.cpp)
drives the editor's sequence (configure, init, bind scene and light,
initProbes, scheduled updates with the hysteresis ramp) and must produce the
same ramp values, atlases and probe states, bit for bit, as the Python
mirror of the same class driving the same sequence.

The compile-and-link check runs without a GPU; the comparison is a GPU
test."""
import os
import subprocess

import numpy as np
import pytest

from vulkanexp_gb300 import abi, build, scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "native", "irradiance_probes_facade.cpp")


def compile_facade(out_dir):
    lib = build.build()
    exe = os.path.join(out_dir, "irradiance_probes_facade")
    libdir = os.path.dirname(lib)
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                    SRC, "-o", exe, "-L", libdir, "-lddgi_gb300", "-Wl,-rpath," + libdir], check=True)
    return exe


def test_facade_compiles_and_links(tmp_path):
    exe = compile_facade(str(tmp_path))
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr


def write_inputs(d, w, updates, per_update, target):
    open(os.path.join(d, "grid.bin"), "wb").write(bytes(w.grid))
    open(os.path.join(d, "light.bin"), "wb").write(bytes(w.light))
    np.array([updates, per_update, np.float32(target).view(np.uint32)], np.uint32).tofile(os.path.join(d, "params.bin"))
    np.stack([w.orientation(k) for k in range(updates + 1)]).astype(np.float32).tofile(os.path.join(d, "orient.bin"))
    sc = w.scene
    for name in ("vertices", "indices", "meshes", "instances", "offsets", "materials"):
        np.ascontiguousarray(getattr(sc, name)).tofile(os.path.join(d, name + ".bin"))


@pytest.mark.gpu
@pytest.mark.parametrize("precision,per_update", [(abi.PRECISION_FP32, 0), (abi.PRECISION_BF16, 50)])
def test_facade_matches_python_mirror(gpu_lib, tmp_path, precision, per_update):
    from vulkanexp_gb300.ddgi import IrradianceProbes

    w = scenes.room_workload(61, n_boxes=60, resolution=(5, 4, 5), rays=64, precision=precision)
    w.grid.hysteresis = 0.3
    updates, target = 24, 0.95
    d = str(tmp_path)
    write_inputs(d, w, updates, per_update, target)
    exe = compile_facade(d)
    r = subprocess.run([exe, d], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr

    p = IrradianceProbes()
    p.GridParameters = w.grid.copy()
    p.ProbesPerUpdate = per_update
    p.TargetHysteresis = target
    p.init(w.grid.extent_min, w.grid.extent_max)
    p.setScene(w.scene)
    p.setLightBuffer(w.light)
    p.initProbes(w.orientation(0))
    ramp = []
    for k in range(updates):
        p.update(w.orientation(k + 1))
        ramp.extend(p.hysteresis()[:2])
    color = p.ctx.get_atlas(abi.ATLAS_COLOR)
    depth = p.ctx.get_atlas(abi.ATLAS_DEPTH)
    states = p.ctx.get_probe_states()
    p.destroy()

    out = np.fromfile(os.path.join(d, "out.bin"), np.uint8)
    n_r, n_c, n_d = 2 * updates * 4, color.nbytes, depth.nbytes
    assert out.size == n_r + n_c + n_d + states.nbytes
    got_ramp = out[:n_r].view(np.float32)
    assert (got_ramp == np.array(ramp, np.float32)).all()
    assert len(set(got_ramp[::2].tolist())) > 3  # the ramp moved
    assert (out[n_r:n_r + n_c].view(np.uint32) == color.view(np.uint32).reshape(-1)).all()
    assert (out[n_r + n_c:n_r + n_c + n_d].view(np.uint32) == depth.view(np.uint32).reshape(-1)).all()
    assert (out[n_r + n_c + n_d:].view(np.uint32) == states).all()
