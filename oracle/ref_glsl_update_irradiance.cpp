// ref_glsl_update_irradiance.cpp — the reference's irradiance update pass
// (src/shaders/probesUpdateIrradiance.comp) on the host.  Test
// infrastructure: built by oracle/build_ref_glsl.py into oracle/_ref/.
#define IRRADIANCE
#define REF_PASS_FN ref_update_irradiance
#define REF_PASS_RES(d) ((d)->color_res)
#define REF_PASS_CHANNELS 4
#include "ref_glsl_update_pass.inc"
