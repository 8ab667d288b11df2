"""Builds oracle/_ref/libref_glsl.so: the reference's own shader code
compiled as C++, for checking the oracle's restatements of it.  The helper
files (src/shaders/common.glsl, ProbeGrid.glsl, irradiance.glsl,
pbrMetallicRoughness.glsl, sky.glsl) compile over oracle/glsl_shim.hpp; the
probe-update compute passes (probesUpdate.glsl as probesUpdateIrradiance.comp
and probesUpdateDepth.comp include it, and probesCopyBorders.comp) compile
over oracle/glsl_compute.hpp, which runs a dispatch's workgroups with one
thread per invocation; the ray-tracing stages (probe trace, probe
classification) over oracle/glsl_rt.hpp; FinalGather.frag once per pixel.
The host-side probe selection (IrradianceProbes::selectProbesToUpdate) is
copied out of src/IrradianceProbes.cpp as written and compiled inside a
stand-in class (oracle/ref_host_select.cpp), the hysteresis ramp block of
update() in a stand-in member function (oracle/ref_host_ramp.cpp), and
genBasis with the reference's vendored GLM (oracle/ref_host_basis.cpp).

Recipe: the files are copied from the reference tree into oracle/_ref/glsl/
with their `#version` and `#extension` lines removed and their resource
declarations -- the only lines C++ cannot take -- rewritten as C++
declarations (`translate` below; statements and function bodies are not
touched), then g++ compiles oracle/ref_glsl_*.cpp, which include them, with
float literals as float (-fsingle-precision-constant, GLSL's rule) and no
contraction.  Test infrastructure: oracle/_ref/ is not part of the product
and is not committed.

    python oracle/build_ref_glsl.py <reference root>
"""
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT, "libref_glsl.so")
SHADERS = ["common.glsl", "ProbeGrid.glsl", "irradiance.glsl", "pbrMetallicRoughness.glsl", "sky.glsl",
           "probesUpdate.glsl", "probesCopyBorders.comp", "traceProbes.rgen", "closesthit.glsl",
           "closesthit_noreflection.rchit", "miss.rmiss", "shadow.rmiss", "rayPayload.glsl", "InstanceMasks.glsl",
           "Lights.glsl", "Vertex.glsl", "Material.glsl", "unpackMaterial.glsl", "probesInit.rgen",
           "probeInitMiss.rmiss", "backfaceTest.rchit", "FinalGather.frag"]
SOURCES = ["ref_glsl_irradiance.cpp", "ref_glsl_pbr.cpp", "ref_glsl_sky.cpp", "ref_glsl_update_irradiance.cpp",
           "ref_glsl_update_depth.cpp", "ref_glsl_copy_borders.cpp", "ref_glsl_trace.cpp", "ref_glsl_closesthit.cpp",
           "ref_glsl_miss.cpp", "ref_glsl_probe_init.cpp", "ref_glsl_final_gather.cpp"]
FORMATS = ("rgba32f", "r11f_g11f_b10f", "rg16f")


def translate(text):
    """GLSL resource declarations as C++ declarations:
    * `#version` / `#extension` lines: removed;
    * a stage input or output `layout(...) in|out T name;`: thread_local
      (one thread per invocation or fragment);
    * `layout(local_size_x = X, local_size_y = Y, local_size_z = Z) in;`:
      the gl_WorkGroupSize constant it defines;
    * a uniform or buffer block without an instance name: its members as
      globals (a runtime-sized array `T name[]` as a pointer `T* name`);
    * a uniform block with an instance name (the push constants): a struct
      of that name and a global of that instance name;
    * `layout(..., <format>) uniform image2D name;`: an image2D of that
      format;
    * `shared T name...;`: a file-scope static (one workgroup runs at a time);
    * a private global `T name;` at file scope: thread_local (one thread per
      invocation)."""
    text = re.sub(r"(?m)^[ \t]*#[ \t]*(version|extension)\b.*$", "", text)
    text = re.sub(r"layout\s*\([^)]*\)\s*(?:in|out)\s+(\w+)\s+(\w+)\s*;", r"thread_local \1 \2;", text)
    text = re.sub(r"layout\s*\(\s*local_size_x\s*=\s*(\d+)\s*,\s*local_size_y\s*=\s*(\d+)\s*,"
                  r"\s*local_size_z\s*=\s*(\d+)\s*\)\s*in\s*;",
                  r"const uvec3 gl_WorkGroupSize = uvec3(\1u, \2u, \3u);", text)

    def block(m):
        members = re.sub(r"(\w+)\s+(\w+)\s*\[\s*\]\s*;", r"\1* \2;", m.group(2))
        if m.group(3):
            return "struct %s {%s} %s;" % (m.group(1), members, m.group(3))
        return members.strip()
    text = re.sub(r"layout\s*\([^)]*\)\s*(?:uniform|buffer)\s+(\w+)\s*\{([^}]*)\}\s*(\w*)\s*;", block, text)

    def image(m):
        fmt = [f.strip() for f in m.group(1).split(",") if f.strip() in FORMATS]
        return "image2D %s(IMG_%s);" % (m.group(2), fmt[0])
    text = re.sub(r"layout\s*\(([^)]*)\)\s*uniform\s+image2D\s+(\w+)\s*;", image, text)
    text = re.sub(r"layout\s*\([^)]*\)\s*uniform\s+(\w+)\s+(\w+)\s*\[\s*\]\s*;", r"\1* \2;", text)
    text = re.sub(r"layout\s*\([^)]*\)\s*uniform\s+(\w+)\s+(\w+)\s*;", r"\1 \2;", text)
    text = re.sub(r"layout\s*\(\s*location\s*=\s*(\d+)\s*\)\s*rayPayloadEXT\s+(\w+)\s+(\w+)\s*;",
                  r"RT_PAYLOAD(\1, \2, \3)", text)
    text = re.sub(r"layout\s*\(\s*location\s*=\s*(\d+)\s*\)\s*rayPayloadInEXT\s+(\w+)\s+(\w+)\s*;",
                  r"RT_PAYLOAD_IN(\1, \2, \3)", text)
    text = re.sub(r"hitAttributeEXT\s+(\w+)\s+(\w+)\s*;", r"RT_HIT_ATTRIBUTE(\1, \2)", text)
    text = re.sub(r"(?m)^([ \t]*)shared\s+", r"\1static ", text)
    text = re.sub(r"(?m)^((?:[iu]?vec[234]|float|int|uint|bool)\s+\w+\s*;)", r"thread_local \1", text)
    return text


def extract_function(text, signature):
    """The definition that starts with `signature` in a C++ source text, up to
    its matching closing brace."""
    start = text.index(signature)
    depth, i = 0, text.index("{", start)
    while True:
        if text[i] == "{":
            depth += 1
        elif text[i] == "}":
            depth -= 1
            if depth == 0:
                return text[start:i + 1] + "\n"
        i += 1


def build(reference_root):
    """Builds the library from the shader files under `reference_root`;
    returns its path, or None when the reference tree is absent."""
    src_dir = os.path.join(reference_root, "src", "shaders")
    if not all(os.path.exists(os.path.join(src_dir, f)) for f in SHADERS):
        return None
    glsl_dir = os.path.join(OUT, "glsl")
    os.makedirs(glsl_dir, exist_ok=True)
    for f in SHADERS:
        with open(os.path.join(src_dir, f)) as fh:
            text = fh.read()
        text = translate(text)
        with open(os.path.join(glsl_dir, f), "w") as fh:
            fh.write(text)
    # the reference's host-side probe selection, its definition as written
    src_out = os.path.join(OUT, "src")
    os.makedirs(src_out, exist_ok=True)
    with open(os.path.join(reference_root, "src", "IrradianceProbes.cpp")) as fh:
        text = fh.read()
    fn = extract_function(text, "uint32_t IrradianceProbes::selectProbesToUpdate()")
    with open(os.path.join(src_out, "selectProbesToUpdate.inc"), "w") as fh:
        fh.write(fn)
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-fsingle-precision-constant", "-ffp-contract=off",
           "-w", "-I", HERE, "-I", glsl_dir, "-I", src_out, "-o", LIB + ".tmp"] + [os.path.join(HERE, s) for s in SOURCES]
    # the hysteresis ramp of update(), the block as written
    a = text.index("	static uint32_t updatedProbes = 0;")
    b = text.index("updatedProbes += probeCount;", a) + len("updatedProbes += probeCount;")
    with open(os.path.join(src_out, "hysteresisRamp.inc"), "w") as fh:
        fh.write(text[a:b] + "\n")
    # and its genBasis, over the reference's vendored GLM
    with open(os.path.join(src_out, "genBasis.inc"), "w") as fh:
        fh.write(extract_function(text, "void genBasis(const glm::vec3& n, glm::vec3& b1, glm::vec3& b2)"))
    # the host functions are plain C++: no single-precision literals there
    for name, extra in (("ref_host_select", []), ("ref_host_ramp", []),
                        ("ref_host_basis", ["-I", os.path.join(reference_root, "ext", "glm")])):
        obj = os.path.join(OUT, name + ".o")
        r = subprocess.run(["g++", "-std=c++17", "-O2", "-fPIC", "-c", "-w", "-ffp-contract=off", "-I", src_out] + extra +
                           ["-o", obj, os.path.join(HERE, name + ".cpp")], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("reference host build failed:\n" + r.stdout + r.stderr)
        cmd.append(obj)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference shader build failed:\n" + r.stdout + r.stderr)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python oracle/build_ref_glsl.py <reference root>")
    path = build(sys.argv[1])
    print(path or "reference shaders not found under %s" % sys.argv[1])
