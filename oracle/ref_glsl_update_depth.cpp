// ref_glsl_update_depth.cpp — the reference's depth update pass
// (src/shaders/probesUpdateDepth.comp) on the host.  Test infrastructure:
// built by oracle/build_ref_glsl.py into oracle/_ref/.
#define DEPTH
#define REF_PASS_FN ref_update_depth
#define REF_PASS_RES(d) ((d)->depth_res)
#define REF_PASS_CHANNELS 2
#include "ref_glsl_update_pass.inc"
