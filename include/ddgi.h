/*
 * ddgi.h — C ABI of the GB300 DDGI irradiance-probe update.
 *
 * This library replaces the probe-update pass of VulkanExp's
 * `IrradianceProbes` class (src/IrradianceProbes.hpp:16-129,
 * src/IrradianceProbes.cpp:12-594) and the GPU programs it drives
 * (src/shaders/traceProbes.rgen, closesthit.glsl with NO_REFLECTION,
 * miss.rmiss, shadow.rmiss, probesUpdate.glsl, probesCopyBorders.comp,
 * probesInit.rgen).  The driver-built Vulkan BLAS/TLAS
 * (src/Renderer.cpp:240-642) is replaced by this library's own trees, built
 * on the GPU: surface-area-heuristic trees with spatial splits (the default,
 * like the driver's PREFER_FAST_TRACE structures) or an LBVH
 * (ddgi_set_build_mode), traversed by CUDA kernels.
 *
 * Conventions
 *  - Every entry point returns a ddgi_status and never throws.
 *  - The context owns its device memory; callers own host arrays and streams.
 *  - A context is not thread-safe; separate contexts are independent.
 *  - Streams are passed as `ddgi_stream` (a cudaStream_t); NULL is the legacy
 *    default stream.
 *  - Host arrays are read during the call only and may be freed afterwards.
 */
#ifndef DDGI_H
#define DDGI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* ddgi_stream; /* == cudaStream_t */
typedef struct ddgi_ctx ddgi_ctx;

typedef enum ddgi_status {
    DDGI_OK = 0,
    DDGI_ERR_INVALID_ARGUMENT = 1, /* bad pointer, size or grid parameter */
    DDGI_ERR_CUDA = 2,             /* a CUDA runtime call failed (see ddgi_last_error) */
    DDGI_ERR_OUT_OF_MEMORY = 3,
    DDGI_ERR_NO_SCENE = 4,         /* update/init before ddgi_scene_build */
    DDGI_ERR_TIMEOUT = 5,          /* ddgi_synchronize gave up waiting */
    DDGI_ERR_DEVICE = 6,           /* a kernel raised its error word (stack overflow, bad index) */
    DDGI_ERR_UNSUPPORTED = 7,      /* valid request this build does not implement */
    DDGI_ERR_IO = 8                /* a checkpoint file cannot be written / read, or does not fit the context */
} ddgi_status;

/* Blend precision of ddgi_update. */
typedef enum ddgi_precision {
    DDGI_PRECISION_FP32 = 0, /* plain form: FP32 SIMT blend, FP32 atlas */
    DDGI_PRECISION_BF16 = 1, /* tcgen05 BF16 contraction, FP32 accumulate, FP16 atlas */
    /* FP32 blend whose stored texels are rounded to the reference's atlas image
     * formats (src/IrradianceProbes.cpp:41, 63): irradiance as
     * B10G11R11_UFLOAT (11-bit red/green, 10-bit blue unsigned floats; alpha
     * reads 1), depth as R16G16_SFLOAT; round to nearest even
     * (ddgi_round_r11/b10/half in ddgi_exact.h).  Texels are kept in the FP32
     * atlas arrays (each stored value is exactly representable in both). */
    DDGI_PRECISION_REFERENCE_FORMAT = 2
} ddgi_precision;

/*
 * Grid parameters.  Mirrors IrradianceProbes::GridInfo
 * (src/IrradianceProbes.hpp:49-60; std140 layout in
 * src/shaders/ProbeGrid.glsl:4-15).  colorRes/depthRes are runtime values here
 * (the reference bakes 8/16 into its shaders); the last word selects the blend
 * precision where the reference has padding.
 */
typedef struct ddgi_grid_desc {
    float extent_min[3];
    float depth_sharpness;   /* exponent of the depth blend weight */
    float extent_max[3];
    float hysteresis;        /* weight of the previous atlas value */
    int32_t resolution[3];   /* probes along x, y, z (each >= 2) */
    uint32_t rays_per_probe; /* 1 .. DDGI_MAX_RAYS_PER_PROBE */
    uint32_t color_res;      /* colour tile side incl. 1-texel border (>= 3) */
    uint32_t depth_res;      /* depth tile side incl. 1-texel border (>= 3) */
    float shadow_bias;
    uint32_t precision;      /* ddgi_precision */
} ddgi_grid_desc;

#define DDGI_MAX_RAYS_PER_PROBE 1024u
/* Limit of probes x rays_per_probe, the rays of one update: ray indices are
 * 32-bit, with headroom for the work counters of the persistent kernels
 * (an update that large needs more than 300 GB of ray and hit buffers). */
#define DDGI_MAX_RAYS_PER_UPDATE 0xFFF00000u

/* Vertex record, 64 bytes.  Same layout as src/vulkan/Vertex.hpp:8-15. */
typedef struct ddgi_vertex {
    float pos[3];
    float color[3];
    float normal[3];
    float tangent[4];
    float uv[2];
    uint32_t padding;
} ddgi_vertex;

/* Material::Properties, 12 words (src/vulkan/Material.hpp:16-25).
 * Texture ids are accepted but textures are not sampled. */
typedef struct ddgi_material {
    float metallic;
    float roughness;
    float base_color[3];
    float emissive[3];
    uint32_t albedo_texture;
    uint32_t normal_texture;
    uint32_t metallic_roughness_texture;
    uint32_t emissive_texture;
} ddgi_material;

/* Renderer::OffsetEntry (src/Renderer.hpp:21-25), indexed by an instance's
 * custom index at shading time (src/shaders/closesthit.glsl:147-155). */
typedef struct ddgi_offset_entry {
    uint32_t material_index;
    uint32_t vertex_offset; /* in vertices */
    uint32_t index_offset;  /* in indices */
} ddgi_offset_entry;

/* One bottom-level structure is built per mesh over its index range
 * (src/Renderer.cpp:272-449).  Indices are relative to vertex_offset. */
typedef struct ddgi_mesh {
    uint32_t vertex_offset;
    uint32_t vertex_count;
    uint32_t index_offset;
    uint32_t index_count; /* multiple of 3 */
} ddgi_mesh;

/* Like VkAccelerationStructureInstanceKHR (src/Renderer.cpp:538-550):
 * object-to-world transform, row-major 3x4; 24-bit custom index (an
 * offset-table entry) and 8-bit visibility mask; the mesh it instances. */
typedef struct ddgi_instance {
    float transform[12];
    uint32_t custom_index; /* low 24 bits used */
    uint32_t mask;         /* low 8 bits used */
    uint32_t mesh_index;
    uint32_t padding;
} ddgi_instance;

/* LightBuffer (src/Light.hpp:6-9): direction points TOWARDS the sun,
 * color.rgb is the sun radiance, color.a the sun brightness factor the
 * atmospheric sky multiplies it by (miss.rmiss:22).  sky.rgb is the constant
 * radiance returned on a miss in the default sky mode (ddgi_set_sky_mode). */
typedef struct ddgi_light {
    float direction[4];
    float color[4];
    float sky[4];
} ddgi_light;

typedef struct ddgi_scene_desc {
    const ddgi_vertex* vertices;
    uint32_t vertex_count;
    const uint32_t* indices;
    uint32_t index_count;
    const ddgi_mesh* meshes;
    uint32_t mesh_count;
    const ddgi_instance* instances;
    uint32_t instance_count;
    const ddgi_offset_entry* offsets;
    uint32_t offset_count;
    const ddgi_material* materials;
    uint32_t material_count;
} ddgi_scene_desc;

/* Closest-hit record of one probe ray (for parity checks).
 * instance == 0xFFFFFFFF marks a miss. */
typedef struct ddgi_hit {
    uint32_t instance;
    uint32_t primitive;
    float t;
    uint32_t backface;
} ddgi_hit;

typedef enum ddgi_atlas_kind {
    DDGI_ATLAS_COLOR = 0, /* RGBA per texel, A = 1 */
    DDGI_ATLAS_DEPTH = 1  /* (mean distance, mean squared distance) per texel */
} ddgi_atlas_kind;

/* Per-stage device times of the last update, in milliseconds, in the order of
 * the reference's five timestamps (src/IrradianceProbes.cpp:441-452):
 * total, trace+shade, blend, border copy, atlas publish; then the part of
 * trace+shade spent in the primary closest-hit traversal. */
typedef struct ddgi_timings {
    float total_ms;
    float trace_ms;
    float blend_ms;
    float border_ms;
    float copy_ms;
    float primary_ms;
} ddgi_timings;

/* How the trace + shade of an update is scheduled.  Both give identical
 * results. */
typedef enum ddgi_pipeline {
    DDGI_PIPELINE_FUSED = 0,     /* one thread per ray: trace, shade, shadow ray */
    DDGI_PIPELINE_WAVEFRONT = 1  /* persistent primary traversal, shading, compacted shadow traversal (default) */
} ddgi_pipeline;

const char* ddgi_status_string(ddgi_status status);
/* Message of the last failing call on this context (never NULL). */
const char* ddgi_last_error(const ddgi_ctx* ctx);

/* IrradianceProbes::init (src/IrradianceProbes.cpp:12-104): validates the
 * grid and allocates the atlases and per-ray buffers on the current device.
 * The atlas starts at zero; probe states start at 1 (ON). */
ddgi_status ddgi_create(const ddgi_grid_desc* grid, ddgi_ctx** out);
ddgi_status ddgi_destroy(ddgi_ctx* ctx);

/* IrradianceProbes::updateUniforms (src/IrradianceProbes.cpp:106-108):
 * replace hysteresis, depth sharpness, shadow bias, rays per probe, extent
 * and precision.  Resolution, colorRes and depthRes must not change. */
ddgi_status ddgi_set_grid(ddgi_ctx* ctx, const ddgi_grid_desc* grid);
ddgi_status ddgi_get_grid(const ddgi_ctx* ctx, ddgi_grid_desc* out);

/* IrradianceProbes::TargetHysteresis (src/IrradianceProbes.hpp:46) and the
 * hysteresis ramp of IrradianceProbes::update (src/IrradianceProbes.cpp:
 * 462-476).  target in [0, 1] switches the ramp on (or changes its target);
 * a negative target switches it off, so the grid's hysteresis is blended as
 * given (the default).  A ramp switched on starts from the grid's hysteresis
 * (GridParameters.hysteresis) with no probes counted.  Every ddgi_update and
 * ddgi_update_scheduled then runs the reference's step on the device before
 * its blend: once a full grid's worth of probes has been refreshed since the
 * last step, the value is either uploaded and then moved a tenth of the way
 * to the target (the reference calls updateUniforms() before the increment,
 * so the blend sees each value one step late) or, within 0.05 of the
 * target, set to the target and uploaded; then the update's probe count is
 * added (for ddgi_update_scheduled, the count selected on the device: no
 * readback).  ddgi_set_grid (updateUniforms) resets both the blended and the
 * host-side value to the new grid's hysteresis; ddgi_init_probes zeroes the
 * host-side value.  The reference keeps the probe counter in a function-static
 * variable shared by every instance; here each context has its own.  Takes
 * effect from the next update on. */
ddgi_status ddgi_set_target_hysteresis(ddgi_ctx* ctx, float target);
/* The ramp's state after the work queued on `stream` (synchronous): the
 * hysteresis the last update blended with (the reference's uniform buffer
 * value), the host-side GridParameters.hysteresis and the probes counted
 * since the last step.  With the ramp off both values are the grid's and the
 * count is 0.  Any pointer may be NULL. */
ddgi_status ddgi_get_hysteresis(ddgi_ctx* ctx, float* blended, float* parameter, uint32_t* counted,
                                ddgi_stream stream);
uint32_t ddgi_probe_count(const ddgi_ctx* ctx);

/* Builds the bottom-level LBVHs (one per mesh) and the top-level LBVH over
 * the instances on `stream`, replacing the Vulkan BLAS/TLAS build
 * (src/Renderer.cpp:272-449, 525-642).  Returns after the build completes. */
ddgi_status ddgi_scene_build(ddgi_ctx* ctx, const ddgi_scene_desc* scene, ddgi_stream stream);

/* IrradianceProbes::setLightBuffer / writeLightDescriptor
 * (src/IrradianceProbes.cpp:323-336). */
ddgi_status ddgi_set_light(ddgi_ctx* ctx, const ddgi_light* light);

/* Radiance of probe rays that miss the scene (src/shaders/miss.rmiss:17-23). */
typedef enum ddgi_sky_mode {
    DDGI_SKY_CONSTANT = 0,  /* the light's sky.rgb (default) */
    /* sky() of src/shaders/sky.glsl:60-127, single-scattering atmosphere seen
     * from the ray origin along the ray, sun from the light's direction,
     * color.rgb and color.a (showSun = true); the final gather's sky pixels
     * use it with brightness 1 and the view direction in position.xyz
     * (FinalGather.frag:56).  Not with ddgi_forward_record / ddgi_backward
     * (the sky radiance is a parameter there) nor in a batch. */
    DDGI_SKY_ATMOSPHERE = 1
} ddgi_sky_mode;
ddgi_status ddgi_set_sky_mode(ddgi_ctx* ctx, ddgi_sky_mode mode);

/* IrradianceProbes::update (src/IrradianceProbes.cpp:426-594).
 * `orientation` is the row-major 3x3 rotation applied to the spherical
 * Fibonacci ray set (the push constant of src/shaders/traceProbes.rgen:36).
 * `probe_list` lists linear probe indices to update; NULL updates all probes
 * in index order.  Work is enqueued on `stream`; the call does not wait. */
ddgi_status ddgi_update(ddgi_ctx* ctx, const float orientation[9], const uint32_t* probe_list,
                        uint32_t probe_count, ddgi_stream stream);

/* The blend + border-copy stage of an update alone (probesUpdate.glsl and
 * probesCopyBorders.comp), fed with caller-provided ray records
 * (r, g, b, depth) per (probe slot, ray) instead of traced ones; uses the
 * context's precision.  `count` = listed probes * rays_per_probe.  No scene
 * is needed.  Synchronous on `stream`. */
ddgi_status ddgi_blend_records(ddgi_ctx* ctx, const float orientation[9], const uint32_t* probe_list,
                               uint32_t probe_count, const float* records, size_t count, ddgi_stream stream);

/* Allocation-free BF16 blend.  This entry point has no counterpart in the
 * reference; it exists for callers that cannot allocate device memory at the
 * time they blend: an engine that reserves its whole device-memory budget up
 * front, or a frame loop that must not call cudaMalloc/cudaFree (they can
 * synchronise the device and stall the frame).  It runs the same blend +
 * border copy + state update as ddgi_blend_records on a BF16 context, but on
 * device buffers the caller owns and without a context:
 *   probe_list  device, probe_count distinct linear probe indices (NULL = all);
 *   records     device, (r, g, b, depth) float4 per (probe slot, ray);
 *   states      device, one uint32 per probe (read and updated);
 *   color/depth device, the FP16 atlases (4 x half / 2 x half per texel);
 *   acc_color/acc_depth device, their FP32 hysteresis accumulators
 *               (float4 / float2 per texel, same layout).
 * Its own working memory (ray-direction table, weight matrices, row sums,
 * error word; about 2 MB) is one fixed __device__ array that every GPU using
 * the library holds until the process exits; requests that would need more
 * (rays_per_probe x texel rows beyond 2 MB of weights, or interior tiles
 * above 16 x 16 texels) return DDGI_ERR_UNSUPPORTED.  Every call looks up
 * that array's device address in the caller's current context
 * (cudaGetSymbolAddress, a host call) and should therefore not be made
 * during a stream capture.  All calls share the
 * array, so calls that overlap on the GPU (other streams, other host threads)
 * race: serialise them.  Synchronous on `stream`; kernel-detected errors
 * (a probe index outside the grid) return DDGI_ERR_DEVICE. */
ddgi_status ddgi_blend_records_noalloc(const ddgi_grid_desc* grid, const float orientation[9],
                                       const uint32_t* probe_list, uint32_t probe_count, const float* records,
                                       uint32_t* states, void* color, void* depth, float* acc_color,
                                       float* acc_depth, ddgi_stream stream);

/* Copies an atlas to host memory as FP32 (RGBA for colour, RG for depth),
 * row-major, width = res*resolution.x*resolution.y, height = res*resolution.z.
 * `bytes` must equal width*height*channels*4.  Synchronous on `stream`. */
ddgi_status ddgi_get_atlas(ddgi_ctx* ctx, ddgi_atlas_kind kind, float* dst, size_t bytes,
                           ddgi_stream stream);
/* Copies an atlas to host memory in its storage format: FP32 texels for an
 * FP32 context, IEEE half texels (4 x half colour, 2 x half depth) for a
 * BF16-blend context, the format a renderer samples (the reference's atlases
 * are 16-bit float images, src/IrradianceProbes.cpp:41, 63).  `bytes` must
 * equal width*height*channels*(4 or 2).  Synchronous on `stream`. */
ddgi_status ddgi_get_atlas_raw(ddgi_ctx* ctx, ddgi_atlas_kind kind, void* dst, size_t bytes, ddgi_stream stream);
/* Replaces an atlas from host FP32 data of the same shape (checkpoint load). */
ddgi_status ddgi_set_atlas(ddgi_ctx* ctx, ddgi_atlas_kind kind, const float* src, size_t bytes,
                           ddgi_stream stream);
/* Atlas checkpoints (no counterpart in the reference, whose atlases live
 * only in GPU images): the context's atlases, for an FP16 (BF16-blend)
 * context also its FP32 hysteresis accumulators, and the probe states,
 * written to / read from a file with a header holding the grid.  Loading
 * needs the same probe resolution, tile sides and precision.  Both wait for
 * `stream`.  File format, little-endian: "DDGIATL1", u32 version (1), u32
 * fp16, the 64-byte ddgi_grid_desc, u32 colour w, h, depth w, h, probe
 * count, 3 reserved words; then colour atlas, depth atlas (FP32 or FP16
 * texels, row-major), [FP32 colour and depth accumulators], u32 states. */
ddgi_status ddgi_atlas_save(ddgi_ctx* ctx, const char* path, ddgi_stream stream);
ddgi_status ddgi_atlas_load(ddgi_ctx* ctx, const char* path, ddgi_stream stream);
ddgi_status ddgi_atlas_dims(const ddgi_ctx* ctx, ddgi_atlas_kind kind, uint32_t* width,
                            uint32_t* height, uint32_t* channels);

/* Ray records of the last update: (r, g, b, depth) per (probe slot, ray),
 * slot-major, as written by src/shaders/traceProbes.rgen:45.  `count` is
 * probe_count * rays_per_probe of that update. */
ddgi_status ddgi_get_ray_records(ddgi_ctx* ctx, float* dst, size_t count, ddgi_stream stream);
/* Closest-hit records of the last update, same order as the ray records.
 * Recorded only when hit recording is on (ddgi_record_hits). */
ddgi_status ddgi_record_hits(ddgi_ctx* ctx, int enable);
ddgi_status ddgi_get_hits(ddgi_ctx* ctx, ddgi_hit* dst, size_t count, ddgi_stream stream);
/* Ray directions of the last update (x, y, z, 1) per ray
 * (src/shaders/traceProbes.rgen:46-47). */
ddgi_status ddgi_get_ray_directions(ddgi_ctx* ctx, float* dst, size_t count);

/* Probe states (0 OFF, 1..8 refresh period) as in ProbeInfo
 * (src/IrradianceProbes.hpp:64-66). */
ddgi_status ddgi_get_probe_states(ddgi_ctx* ctx, uint32_t* dst, size_t count, ddgi_stream stream);
ddgi_status ddgi_set_probe_states(ddgi_ctx* ctx, const uint32_t* src, size_t count,
                                  ddgi_stream stream);

/* Device pointers of the current atlases (FP32 form: float4 colour and
 * float2 depth; BF16 form: half4 colour and half2 depth), for zero-copy
 * consumers.  Valid until the next ddgi_update, ddgi_set_grid or destroy. */
ddgi_status ddgi_atlas_device_ptr(const ddgi_ctx* ctx, ddgi_atlas_kind kind, void** ptr);

/* Closest-hit (any_hit = 0) or any-hit (any_hit = 1) queries of n world-space
 * rays against the built scene, with t in [tmin, tmax] and an instance mask:
 * the traceRayEXT calls of src/shaders/traceProbes.rgen:43 and
 * src/shaders/closesthit.glsl:270-281, exposed for parity checks.  Host
 * arrays: origins/dirs 3*n floats, hits n records, barycentrics 2*n floats
 * (may be NULL).  Synchronous on `stream`. */
ddgi_status ddgi_trace_rays(ddgi_ctx* ctx, const float* origins, const float* dirs, uint32_t n, float tmin,
                            float tmax, uint32_t mask, int any_hit, ddgi_hit* hits, float* barycentrics,
                            ddgi_stream stream);

/* Measurement: runs the trace + shade of one update (no blend; atlas and
 * probe states untouched) with fetch counters, and returns for the primary
 * (closest-hit) rays out[0] inner-node fetches (64 B each), out[1] triangle
 * tests (48 B each), out[2] instance entries (64 B each), out[3] rays;
 * out[4] shading bytes (hit data, atlas texels of the bounce lookups, ray
 * record); out[5..8] the same four counts for the shadow (any-hit) rays;
 * out[9], out[10] the part of out[0], out[5] in the top-level tree.
 * Synchronous on `stream`. */
ddgi_status ddgi_count_fetches(ddgi_ctx* ctx, const float orientation[9], const uint32_t* probe_list,
                               uint32_t probe_count, uint64_t out[11], ddgi_stream stream);

/* Sizes of the built scene's trees.  node_count binary nodes (the mesh
 * trees in mesh order, then the top level), tri_refs triangle references
 * in leaf order, the deepest mesh tree and the top level's depth (inner
 * nodes on the longest root-to-leaf path), the builder, and the device time
 * of the GPU fast-trace mesh-tree build (0 for the other builders). */
typedef struct ddgi_scene_info {
    uint64_t node_count;
    uint64_t tri_refs;
    uint32_t depth_blas, depth_tlas;
    uint32_t build_mode;
    float tree_build_ms;
} ddgi_scene_info;
ddgi_status ddgi_get_scene_info(const ddgi_ctx* ctx, ddgi_scene_info* out);
/* Copies the built trees to host arrays (for tests): up to node_capacity
 * nodes of 64 bytes (child boxes and references, the library's node
 * layout) and up to tri_capacity triangles of 48 bytes in leaf order
 * (v0 xyz + the mesh-local triangle index as bits, v1, v2); NULL skips an
 * array.  Synchronous on `stream`. */
ddgi_status ddgi_read_trees(ddgi_ctx* ctx, void* nodes, uint64_t node_capacity, void* tris, uint64_t tri_capacity,
                            ddgi_stream stream);

/* Replaces the material table of the built scene (same count), e.g. new
 * albedos, without rebuilding the acceleration structures. */
ddgi_status ddgi_set_materials(ddgi_ctx* ctx, const ddgi_material* materials, uint32_t count);

/* Differentiation (FP32 form, all probes).  Runs K updates from the current
 * atlas, with orientations K x 9, and records what the reverse pass needs:
 * every ray's closest hit and shadow result (the hit set is then held fixed)
 * and an atlas checkpoint every `checkpoint_every` updates.  The atlas ends
 * as after K ordinary updates.  DDGI_ERR_UNSUPPORTED for a BF16 or
 * reference-format context, the atmospheric sky or a hysteresis ramp
 * (the reverse pass differentiates the grid's fixed hysteresis). */
ddgi_status ddgi_forward_record(ddgi_ctx* ctx, uint32_t K, const float* orientations, uint32_t checkpoint_every,
                                ddgi_stream stream);
/* Reverse pass of the last ddgi_forward_record: given dL/d(colour atlas
 * after the K updates) (host, FP32 RGBA per texel, A ignored, `bytes` = the
 * colour atlas size), returns dL/d albedo (material_count x 3), dL/d sun
 * radiance and dL/d sky radiance, carried back through every update's blend,
 * hysteresis, shading and bounce lookup into the previous atlas.  Atlases
 * between checkpoints are recomputed from the recorded hits.  The context's
 * atlas is not modified.  Synchronous on `stream`. */
ddgi_status ddgi_backward(ddgi_ctx* ctx, const float* dL_dcolor, size_t bytes, float* grad_albedo, float grad_sun[3],
                          float grad_sky[3], ddgi_stream stream);

/* Moves instances: Renderer::updateAccelerationStructureInstances +
 * updateTLAS (src/Renderer.cpp:671-742).  `transforms` = count new
 * object-to-world transforms (row-major 3x4) for the instances `ids` (NULL:
 * instances 0 .. count-1).  rebuild = 0: the top-level tree keeps its
 * topology and its boxes are recomputed bottom-up on the device (the
 * reference's UPDATE-mode build); rebuild = 1: the top-level tree is built
 * again over the new instance boxes.  Mesh trees are not touched.  Ordered
 * on `stream`; a batch made from this context must be made again. */
ddgi_status ddgi_update_instances(ddgi_ctx* ctx, const uint32_t* ids, const float* transforms, uint32_t count,
                                  int rebuild, ddgi_stream stream);

/* ---- Probe classification and adaptive schedule -------------------------
 * IrradianceProbes::initProbes (src/IrradianceProbes.cpp:357-394,
 * src/shaders/probesInit.rgen:31-64): classifies every probe from 512 rays
 * (orientation x spherical-Fibonacci direction i of a raysPerProbe-point set,
 * i = 0..511, as the shader does), closest hits among instances with mask
 * bit 0 set, t in [0.01, 1.5 |cell|]: a probe with more than raysPerProbe / 2
 * back-face hits closer than |cell| becomes OFF (state 0, skipped by the
 * updates and by the bounce lookup), else a probe with such a hit within one
 * cell on every axis gets state 1 (refreshed every update), else 8.
 * Synchronous.  Like the reference (src/IrradianceProbes.cpp:357-358), it
 * zeroes the hysteresis ramp's host-side value when the ramp is on
 * (ddgi_set_target_hysteresis); the blended value and the grid stay as they
 * are. */
ddgi_status ddgi_init_probes(ddgi_ctx* ctx, const float orientation[9], ddgi_stream stream);
/* ddgi_update over the probes selectProbesToUpdate
 * (src/IrradianceProbes.cpp:396-424) picks, chosen on the device with no
 * host readback: visiting probes cyclically from where the previous
 * selection stopped, probe i is refreshed when state s != 0 and
 * (i + loop) % s == 0 (loop counts the visit's wraps); max_probes > 0 stops
 * the visit after that many (ProbesPerUpdate), 0 = no cap.  The selection
 * and the schedule state stay on the device; the trace and blend read the
 * selected count there.  Asynchronous like ddgi_update; always the wavefront
 * trace.  Ray/hit records hold the selected probes first, in list order. */
ddgi_status ddgi_update_scheduled(ddgi_ctx* ctx, const float orientation[9], uint32_t max_probes, ddgi_stream stream);
/* The last selection (count, list in visit order) and the schedule state
 * (offset, loop index); any pointer may be NULL.  Synchronous. */
ddgi_status ddgi_get_schedule(ddgi_ctx* ctx, uint32_t* count, uint32_t* offset, uint32_t* loop, uint32_t* list,
                              size_t list_capacity, ddgi_stream stream);
/* Sets the schedule state (a new context starts at offset 0, loop 0). */
ddgi_status ddgi_set_schedule(ddgi_ctx* ctx, uint32_t offset, uint32_t loop, ddgi_stream stream);

/* ---- Final gather (the atlas's consumer) --------------------------------
 * src/shaders/FinalGather.frag:39-80 as a headless pass over a G-buffer in
 * device memory (all arrays width x height, tightly packed, row-major). */
typedef struct ddgi_gbuffer {
    const float* position_depth;   /* float4: world position, depth (<= 0: no geometry, sky) */
    const float* normal_metalness; /* float4: normal (normalised here), metalness */
    const float* albedo_roughness; /* float4: albedo rgb, roughness */
    const float* emissive;         /* float4: emissive rgb */
    const float* direct_light;     /* float: the sun's visibility (the reference's direct-light .r) */
    const float* reflection;       /* float4: the reflection pass at this pixel; NULL = none */
    uint32_t width, height;
} ddgi_gbuffer;
/* color_out (device, float4 per pixel) = direct * GGX sun + mix(0.004,
 * albedo, metal) * reflection + sampleProbes(position, normal, view) *
 * albedo * 0.996 * (1 - metal) + emissive, or the sky radiance on a miss;
 * view = normalize(camera_origin - position).  Reads the context's current
 * atlas and probe states.  Asynchronous on `stream`. */
ddgi_status ddgi_final_gather(ddgi_ctx* ctx, const ddgi_gbuffer* gbuffer, const float camera_origin[3],
                              float* color_out, ddgi_stream stream);

/* ---- Launch tuning of the persistent traversals -------------------------
 * Results do not depend on these; speed does. */
typedef struct ddgi_trace_tuning {
    uint32_t rays_per_warp; /* 0: each warp traces 32 rays of one probe, probes in index order (default);
                               n = 1, 2, 4, 8, 16, 32 (n dividing rays_per_probe): each warp traces n
                               consecutive directions of the octant-binned ray order from 32 / n neighbouring
                               probes (Morton order of the grid); used when all probes are updated */
    uint32_t refill_lanes;  /* a warp requests new rays once this many lanes are idle (1..32, default 8) */
    uint32_t smem_stack;    /* traversal-stack entries per thread in shared memory, deeper ones in local
                               memory; 0 = the whole stack in shared memory (default) */
    uint32_t ctas_per_sm;   /* persistent CTAs per SM; 0 = as many as fit (default) */
    uint32_t node_width;    /* 2: binary nodes (default), 8: eight-wide quantised nodes collapsed from the binary trees */
    uint32_t straggler_lanes; /* a warp leaves its node-search loop to test the leaves its lanes hold once at
                                 most this many lanes still search for one (0..31, default 10; 0: wait for
                                 every lane, the plain while-while traversal) */
} ddgi_trace_tuning;
ddgi_status ddgi_set_trace_tuning(ddgi_ctx* ctx, const ddgi_trace_tuning* tuning);
/* Most triangles per leaf of the mesh trees built by the next
 * ddgi_scene_build (1..8, default 2). */
ddgi_status ddgi_set_leaf_size(ddgi_ctx* ctx, uint32_t max_triangles);
/* Tree builder of the next ddgi_scene_build (mesh trees and top level) and
 * of ddgi_update_instances' top-level rebuilds.  Hits do not depend on it.
 *   DDGI_BUILD_FAST_TRACE (default): surface-area-heuristic trees with
 *     spatial splits built on the GPU (the reference's PREFER_FAST_TRACE
 *     structures, src/Renderer.cpp:334);
 *   DDGI_BUILD_FAST_BUILD: linear BVHs built on the GPU (PREFER_FAST_BUILD,
 *     src/Renderer.cpp:364);
 *   DDGI_BUILD_FAST_TRACE_HOST: the same trees as DDGI_BUILD_FAST_TRACE,
 *     built on the host threads. */
typedef enum ddgi_build_mode {
    DDGI_BUILD_FAST_TRACE = 0,
    DDGI_BUILD_FAST_BUILD = 1,
    DDGI_BUILD_FAST_TRACE_HOST = 2
} ddgi_build_mode;
ddgi_status ddgi_set_build_mode(ddgi_ctx* ctx, ddgi_build_mode mode);
/* Spatial splits of the fast-trace mesh trees built by the next
 * ddgi_scene_build: a node whose object split leaves children overlapping by
 * more than `overlap` of the tree root's surface area also tries splitting
 * its triangles by a plane (they are then referenced on both sides).  0
 * turns them off; default 0.001 (smaller: faster traversal, slower build and
 * more triangle references).  Hits do not depend on it. */
ddgi_status ddgi_set_spatial_splits(ddgi_ctx* ctx, float overlap);

/* ---- Failure-detection test hooks ---------------------------------------
 * No counterpart in the reference (its fence waits use UINT64_MAX).  Every
 * device-side wait of this library is bounded: the tensor-core blend gives
 * up on a completion that does not come within 0.5 s, releases its tensor
 * memory, and the next ddgi_synchronize / ddgi_get_* call returns
 * DDGI_ERR_DEVICE ("device wait timed out"); the context stays usable.
 * DDGI_FAULT_STALL_TENSOR_WAIT makes the next BF16 blend issue no
 * tensor-core work, so its completion wait runs out (one-shot). */
enum { DDGI_FAULT_STALL_TENSOR_WAIT = 1u };
ddgi_status ddgi_inject_fault(ddgi_ctx* ctx, uint32_t faults);
ddgi_status ddgi_get_trace_tuning(const ddgi_ctx* ctx, ddgi_trace_tuning* out);
/* Times candidate tunings on updates of all probes with the given
 * orientation (`reps` timed updates each, coordinate descent), keeps the
 * fastest trace (primary + shading + shadow rays) and writes it to *chosen
 * (may be NULL).  The atlases, accumulators, probe states, the adaptive
 * schedule's position and the hysteresis ramp's state are restored
 * afterwards.  Synchronous. */
ddgi_status ddgi_autotune(ddgi_ctx* ctx, const float orientation[9], uint32_t reps, ddgi_stream stream,
                          ddgi_trace_tuning* chosen);

/* ---- Batched update of many probe volumes ------------------------------
 * No single counterpart in the reference, which updates one IrradianceProbes
 * volume per call (src/IrradianceProbes.cpp:426-594); a batch runs that
 * update for several contexts ("volumes") at once.  Each volume keeps its own
 * grid, scene, light, precision and atlases.  The volumes are ordered by
 * ray count and split into up to four groups, run one after another
 * (smallest first, so small volumes finish early); a group's update is one
 * persistent work-queue traversal launch over the primary rays of all its
 * volumes, one shading launch, one persistent shadow-ray launch, and one
 * blend launch per precision (FP32 SIMT, BF16 tensor core).  The whole
 * sequence is captured once into a CUDA graph and replayed per update.  The
 * result of every volume equals ddgi_update of that volume alone over all
 * its probes.  Volumes with the atmospheric sky (ddgi_set_sky_mode) or a
 * hysteresis ramp (ddgi_set_target_hysteresis) are not batched:
 * ddgi_batch_update returns DDGI_ERR_UNSUPPORTED for them.
 *
 * ddgi_batch_create copies the volumes' acceleration structures into one
 * node/triangle/instance arena, so every volume needs a built scene at that
 * point and a scene rebuilt later needs a new batch (ddgi_batch_update then
 * returns DDGI_ERR_INVALID_ARGUMENT); light and material changes reach the
 * next update.  Ray records and hit records of the volumes are not written by
 * batch updates.  A batch borrows its contexts: destroy it first. */
typedef struct ddgi_batch ddgi_batch;

/* Launch parameters of a batch (ddgi_batch_autotune picks them). */
typedef struct ddgi_batch_tuning {
    uint32_t trace_ctas_per_sm; /* persistent traversal CTAs per SM; 0 = as many as fit */
    uint32_t refill_lanes;      /* a warp requests new rays once this many lanes are idle (1..32) */
    uint32_t smem_stack;        /* traversal-stack entries per thread in shared memory, deeper ones
                                   in local memory; 0 = the whole stack in shared memory */
    uint32_t blend_threads;     /* FP32 blend: 0 = weights computed once per update and shared by tiles of
                                   probes (default); 32..256 (multiple of 32) = one block of this many
                                   threads per probe computing its weights per texel */
    uint32_t rays_per_warp;     /* as in ddgi_trace_tuning, per volume (values a volume's ray count
                                   does not allow fall back to 0 for that volume) */
    uint32_t node_width;        /* as in ddgi_trace_tuning */
    uint32_t straggler_lanes;   /* as in ddgi_trace_tuning */
} ddgi_batch_tuning;

ddgi_status ddgi_batch_create(ddgi_ctx* const* volumes, uint32_t count, ddgi_stream stream, ddgi_batch** out);
ddgi_status ddgi_batch_destroy(ddgi_batch* batch);
const char* ddgi_batch_last_error(const ddgi_batch* batch);
/* Primary rays of one batch update (sum over the volumes of probes x rays). */
uint64_t ddgi_batch_ray_count(const ddgi_batch* batch);
ddgi_status ddgi_batch_get_tuning(const ddgi_batch* batch, ddgi_batch_tuning* out);
ddgi_status ddgi_batch_set_tuning(ddgi_batch* batch, const ddgi_batch_tuning* tuning);
/* Graph replay (default, enable = 1) or plain stream launches (0). */
ddgi_status ddgi_batch_use_graph(ddgi_batch* batch, int enable);
/* One update of every volume; `orientations` = count x 9 row-major ray-set
 * rotations, one per volume.  Waits for the previous batch update's inputs to
 * be consumed, then enqueues on `stream` and returns. */
ddgi_status ddgi_batch_update(ddgi_batch* batch, const float* orientations, ddgi_stream stream);
/* Waits for `stream` (poll, timeout_ms < 0 = forever), then checks the
 * batch's device error word. */
ddgi_status ddgi_batch_synchronize(ddgi_batch* batch, ddgi_stream stream, int timeout_ms);
/* After a synchronised update: per volume, milliseconds from the start of
 * the update to the end of the volume's last blend work item. */
ddgi_status ddgi_batch_completion_ms(ddgi_batch* batch, float* ms, uint32_t count);
/* Times candidate tunings on updates with the given orientations (`reps`
 * timed updates each, coordinate descent over the four parameters), keeps
 * the fastest and writes it to *chosen (may be NULL).  The volumes' atlases,
 * accumulators and probe states are restored afterwards.  Synchronous. */
ddgi_status ddgi_batch_autotune(ddgi_batch* batch, const float* orientations, uint32_t reps, ddgi_stream stream,
                                ddgi_batch_tuning* chosen);

/* Waits for `stream` with a timeout (poll), then checks the device error word.
 * timeout_ms < 0 waits forever. */
ddgi_status ddgi_synchronize(ddgi_ctx* ctx, ddgi_stream stream, int timeout_ms);
ddgi_status ddgi_get_timings(const ddgi_ctx* ctx, ddgi_timings* out);
ddgi_status ddgi_set_pipeline(ddgi_ctx* ctx, ddgi_pipeline pipeline);
/* Enables per-stage CUDA-event timing of updates (off by default). */
ddgi_status ddgi_enable_timing(ddgi_ctx* ctx, int enable);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* DDGI_H */
