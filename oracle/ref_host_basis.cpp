// ref_host_basis.cpp — the reference's genBasis (src/IrradianceProbes.cpp:
// 347-355), the ray-set rotation's basis, compiled from its own source text
// with the reference's vendored GLM: oracle/build_ref_glsl.py copies the
// function's definition into oracle/_ref/src/genBasis.inc.  Test
// infrastructure: built into oracle/_ref/libref_glsl.so.
#include <glm/glm.hpp>

#include "genBasis.inc"

extern "C" void ref_gen_basis(const float* n, float* b1, float* b2) {
    glm::vec3 x, y;
    genBasis(glm::vec3(n[0], n[1], n[2]), x, y);
    for (int k = 0; k < 3; ++k) b1[k] = x[k], b2[k] = y[k];
}
