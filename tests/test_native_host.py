"""Host code under AddressSanitizer, UndefinedBehaviorSanitizer and ThreadSanitizer, no GPU:

* the spatial-split tree builder (vulkanexp_gb300/csrc/sbvh.cu) through
  tests/native/sbvh_check.cu;
* the SAH tree builder (vulkanexp_gb300/csrc/sah.cu) through a structural
  check (tests/native/sah_check.cu) over random, coincident, flat and
  NaN/infinite primitive boxes, every leaf size;
* the REPEAT texel-index wrap of the atlas lookups (tests/native/wrap_check.cu);
* the CPU checker (oracle/ddgi_oracle.cpp) on a small room: trace, update
  (FP32 and FP64), probe classification and final gather, loaded into a
  Python process with the ASan runtime preloaded;
* under ThreadSanitizer: the checker's worker pool and parallel loops (the
  TSan runtime preloaded the same way), and the host tree builders' subtree
  threads (sah_check, sbvh_check with inputs large enough to spawn them).

Any sanitizer report aborts the child process, which fails the test."""
import os
import subprocess
import sys
import textwrap

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SAN = ["-fsanitize=address", "-fsanitize=undefined", "-fno-sanitize-recover=all", "-fno-omit-frame-pointer", "-g",
       "-O1"]
ENV = {"ASAN_OPTIONS": "detect_leaks=0:abort_on_error=1", "UBSAN_OPTIONS": "halt_on_error=1:print_stacktrace=1"}


def _have(tool):
    return subprocess.run(["which", tool], capture_output=True).returncode == 0


def _runtime(name):
    p = subprocess.run(["gcc", "-print-file-name=%s" % name], capture_output=True, text=True).stdout.strip()
    return p if os.path.isabs(p) and os.path.exists(p) else None


def test_sah_builder_under_sanitizers(tmp_path):
    from vulkanexp_gb300 import build

    nvcc = build.nvcc()
    if not (os.path.exists(nvcc) or _have(nvcc)) or _runtime("libasan.so") is None:
        pytest.skip("nvcc or the ASan runtime is missing")
    flags = ["-std=c++17"] + build.ARCH + ["--expt-relaxed-constexpr"]
    for f in SAN[:4] + ["-ffp-contract=off"]:
        flags += ["-Xcompiler", f]
    flags += ["-g", "-O1"]
    objs = []
    for src in ("tests/native/sah_check.cu", "vulkanexp_gb300/csrc/sah.cu"):
        o = str(tmp_path / (os.path.basename(src) + ".o"))
        subprocess.check_call([nvcc] + flags + ["-c", os.path.join(ROOT, src), "-o", o])
        objs.append(o)
    exe = str(tmp_path / "sah_check")
    cudart = os.path.join(os.path.dirname(os.path.dirname(nvcc)), "lib64")
    subprocess.check_call(["g++", "-fsanitize=address", "-fsanitize=undefined"] + objs +
                          ["-L" + cudart, "-lcudart_static", "-ldl", "-lrt", "-pthread", "-o", exe])
    r = subprocess.run([exe], capture_output=True, text=True, env=dict(os.environ, **ENV), timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    assert "all ok" in r.stdout


def test_spatial_split_builder_under_sanitizers(tmp_path):
    """tests/native/sbvh_check.cu: references, leaf ranges, depth, and
    conservativeness at sample points of every triangle, for overlapping box
    soups (several overlap thresholds, leaf sizes) and a height field."""
    from vulkanexp_gb300 import build

    nvcc = build.nvcc()
    if not (os.path.exists(nvcc) or _have(nvcc)) or _runtime("libasan.so") is None:
        pytest.skip("nvcc or the ASan runtime is missing")
    flags = ["-std=c++17"] + build.ARCH + ["--expt-relaxed-constexpr"]
    for f in SAN[:4] + ["-ffp-contract=off"]:
        flags += ["-Xcompiler", f]
    flags += ["-g", "-O1"]
    objs = []
    for src in ("tests/native/sbvh_check.cu", "vulkanexp_gb300/csrc/sbvh.cu"):
        o = str(tmp_path / (os.path.basename(src) + ".o"))
        subprocess.check_call([nvcc] + flags + ["-c", os.path.join(ROOT, src), "-o", o])
        objs.append(o)
    exe = str(tmp_path / "sbvh_check")
    cudart = os.path.join(os.path.dirname(os.path.dirname(nvcc)), "lib64")
    subprocess.check_call(["g++", "-fsanitize=address", "-fsanitize=undefined"] + objs +
                          ["-L" + cudart, "-lcudart_static", "-ldl", "-lrt", "-pthread", "-o", exe])
    r = subprocess.run([exe], capture_output=True, text=True, env=dict(os.environ, **ENV), timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    assert "all ok" in r.stdout


def test_texel_wrap_under_sanitizers(tmp_path):
    """tests/native/wrap_check.cu: the REPEAT texel-index wrap of the atlas
    lookups equals the remainder form for every index it can get."""
    from vulkanexp_gb300 import build

    nvcc = build.nvcc()
    if not (os.path.exists(nvcc) or _have(nvcc)) or _runtime("libasan.so") is None:
        pytest.skip("nvcc or the ASan runtime is missing")
    flags = ["-std=c++17"] + build.ARCH + ["--expt-relaxed-constexpr"]
    for f in SAN[:4]:
        flags += ["-Xcompiler", f]
    flags += ["-g", "-O1"]
    o = str(tmp_path / "wrap_check.o")
    subprocess.check_call([nvcc] + flags + ["-c", os.path.join(ROOT, "tests/native/wrap_check.cu"), "-o", o])
    exe = str(tmp_path / "wrap_check")
    cudart = os.path.join(os.path.dirname(os.path.dirname(nvcc)), "lib64")
    subprocess.check_call(["g++", "-fsanitize=address", "-fsanitize=undefined", o,
                           "-L" + cudart, "-lcudart_static", "-ldl", "-lrt", "-pthread", "-o", exe])
    r = subprocess.run([exe], capture_output=True, text=True, env=dict(os.environ, **ENV), timeout=300)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    assert "all ok" in r.stdout


SCRIPT = textwrap.dedent("""
    import numpy as np
    from oracle.oracle import Oracle, zero_atlas
    from vulkanexp_gb300 import abi, scenes
    w = scenes.room_workload(61, n_boxes=30, resolution=(3, 3, 3), rays=32)
    o = Oracle(w.scene)
    rng = np.random.default_rng(2)
    orig = rng.uniform(-1, 11, size=(500, 3)).astype(np.float32)
    d = rng.normal(size=(500, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    for any_hit in (False, True):
        o.trace(orig, d, 0.01, 100.0, 0xFF, any_hit)
    st = np.ones(w.grid.probe_count(), np.uint32)
    for fp64 in (False, True):
        c, dd = zero_atlas(w.grid, fp64=fp64)
        o.update(w.grid, w.light, w.orientation(0), c, dd, st, fp64=fp64)
        o.update(w.grid, w.light, w.orientation(1), c, dd, st, fp64=fp64)
    o.init_probes(w.grid, w.orientation(0))
    c, dd = zero_atlas(w.grid)
    o.update(w.grid, w.light, w.orientation(0), c, dd, st)
    n = 64
    gb = {"position_depth": np.column_stack([rng.uniform(0, 10, (n, 3)), np.ones(n)]),
          "normal_metalness": np.column_stack([rng.normal(size=(n, 3)), rng.uniform(0, 1, n)]),
          "albedo_roughness": np.column_stack([rng.uniform(0, 1, (n, 3)), rng.uniform(0.1, 1, n)]),
          "emissive": np.zeros((n, 4)), "direct_light": np.ones(n), "reflection": None}
    gb = {k: None if v is None else v.astype(np.float32) for k, v in gb.items()}
    Oracle.final_gather(w.grid, w.light, st, c, dd, gb, (5, 3, 12))
    print("oracle ok")
""")


def test_oracle_under_sanitizers(tmp_path):
    asan = _runtime("libasan.so")
    if asan is None:
        pytest.skip("the ASan runtime is missing")
    lib = str(tmp_path / "libddgi_oracle_san.so")
    subprocess.check_call(["g++", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-pthread"] +
                          SAN + ["-o", lib, os.path.join(ROOT, "oracle", "ddgi_oracle.cpp")])
    env = dict(os.environ, **ENV)
    env.update({"LD_PRELOAD": asan, "DDGI_ORACLE_LIB": lib, "PYTHONPATH": ROOT})
    r = subprocess.run([sys.executable, "-c", SCRIPT], capture_output=True, text=True, env=env, cwd=ROOT,
                       timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    assert "oracle ok" in r.stdout


TSAN_SCRIPT = textwrap.dedent("""
    import numpy as np
    from oracle.oracle import Oracle, zero_atlas
    from vulkanexp_gb300 import scenes
    w = scenes.room_workload(62, n_boxes=30, resolution=(4, 3, 4), rays=32)
    for threads in (4, 3):  # two pools of the same process
        o = Oracle(w.scene, threads=threads)
        st = np.ones(w.grid.probe_count(), np.uint32)
        c, dd = zero_atlas(w.grid)
        for k in range(2):
            o.update(w.grid, w.light, w.orientation(k), c, dd, st)
        o.init_probes(w.grid, w.orientation(0))
        Oracle.blend(w.grid, w.orientation(0), np.zeros((w.grid.probe_count(), 32, 4), np.float32), c, dd, st,
                     threads=threads)
        o.close()
    print("oracle ok")
""")


def test_oracle_worker_pool_under_thread_sanitizer(tmp_path):
    # the checker's worker pool (task queue, futures, one pool per worker
    # count) and the parallel loops over it, with ThreadSanitizer preloaded
    tsan = _runtime("libtsan.so")
    if tsan is None:
        pytest.skip("the ThreadSanitizer runtime is missing")
    lib = str(tmp_path / "libddgi_oracle_tsan.so")
    subprocess.check_call(["g++", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-pthread",
                           "-fsanitize=thread", "-g", "-O1", "-o", lib, os.path.join(ROOT, "oracle", "ddgi_oracle.cpp")])
    env = dict(os.environ)
    env.update({"LD_PRELOAD": tsan, "DDGI_ORACLE_LIB": lib, "PYTHONPATH": ROOT, "TSAN_OPTIONS": "halt_on_error=1",
                "OPENBLAS_NUM_THREADS": "1", "OMP_NUM_THREADS": "1"})
    r = subprocess.run([sys.executable, "-c", TSAN_SCRIPT], capture_output=True, text=True, env=env, cwd=ROOT,
                       timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    assert "oracle ok" in r.stdout


@pytest.mark.parametrize("check,sources,args", [
    # 40,000 boxes: subtrees above 16,384 primitives go to other threads
    ("sah_check", ("tests/native/sah_check.cu", "vulkanexp_gb300/csrc/sah.cu"), []),
    # a 14,400-triangle box soup and a 20,000-triangle height field, above
    # the 8,192 references that send a subtree to another thread
    ("sbvh_check", ("tests/native/sbvh_check.cu", "vulkanexp_gb300/csrc/sbvh.cu"), ["threads"]),
])
def test_host_tree_builders_under_thread_sanitizer(tmp_path, check, sources, args):
    """The host tree builders build subtrees on their own threads (four in
    these checks); ThreadSanitizer watches the shared node and reference
    arrays they fill."""
    from vulkanexp_gb300 import build

    nvcc = build.nvcc()
    if not (os.path.exists(nvcc) or _have(nvcc)) or _runtime("libtsan.so") is None:
        pytest.skip("nvcc or the ThreadSanitizer runtime is missing")
    flags = ["-std=c++17"] + build.ARCH + ["--expt-relaxed-constexpr", "-Xcompiler", "-fsanitize=thread",
                                           "-Xcompiler", "-ffp-contract=off", "-g", "-O1"]
    objs = []
    for src in sources:
        o = str(tmp_path / (os.path.basename(src) + ".o"))
        subprocess.check_call([nvcc] + flags + ["-c", os.path.join(ROOT, src), "-o", o])
        objs.append(o)
    exe = str(tmp_path / check)
    cudart = os.path.join(os.path.dirname(os.path.dirname(nvcc)), "lib64")
    subprocess.check_call(["g++", "-fsanitize=thread"] + objs +
                          ["-L" + cudart, "-lcudart_static", "-ldl", "-lrt", "-pthread", "-o", exe])
    r = subprocess.run([exe] + args, capture_output=True, text=True,
                       env=dict(os.environ, TSAN_OPTIONS="halt_on_error=1"), timeout=900)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    assert "all ok" in r.stdout
