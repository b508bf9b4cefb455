/* tracer_abi.h - C ABI of the GB300 (sm_103a) path tracer.
 *
 * Drop-in for the compute dispatch of stickyfingies/vk-renderer:
 *   Source/GraphicsDevice.cpp:796-822   scene SSBO creation and upload
 *                                       -> tracer_upload_scene
 *   Source/GraphicsDevice.cpp:986-1131  compute descriptors, pipeline,
 *                                       96-byte push-constant range
 *                                       -> tracer_create
 *   Source/GraphicsDevice.cpp:1254-1266 bind + vkCmdPushConstants(FrameData)
 *                                       + vkCmdDispatch(res/16, res/16, 1)
 *                                       -> tracer_trace
 *   Fullscreen.frag sampling the image  -> tracer_readback / tracer_device_image
 * The kernel that runs is the CUDA restatement of Assets/Tracer.comp.
 *
 * Conventions: every call returns an int status (TRACER_OK = 0, errors < 0)
 * and records a message for tracer_last_error.  Host pointers passed in are
 * copied before the call returns; the caller keeps ownership.  A context is
 * not thread-safe (the reference drives its device from one thread,
 * Source/Main.cpp:148-196); separate contexts may be used from separate
 * threads.  Structs below keep the reference's std430 layouts byte for byte.
 */
#ifndef TRACER_ABI_H
#define TRACER_ABI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------ status codes
 * The first three mirror GraphicsDevice::Error (Include/GraphicsDevice.h:46-52),
 * whose SUCCESS is TRACER_OK. */
#define TRACER_OK 0
#define TRACER_ERR_NO_SUITABLE_GPU (-1)     /* no CUDA device of the right kind */
#define TRACER_ERR_NO_SUITABLE_SURFACE (-2) /* image size / AOV cannot be produced */
#define TRACER_ERR_UNKNOWN (-3)
#define TRACER_ERR_INVALID_ARG (-4)
#define TRACER_ERR_OOM (-5)
#define TRACER_ERR_TIMEOUT (-6)             /* a bounded wait for the GPU ran out */
#define TRACER_ERR_TRAVERSAL_LIMIT (-7)     /* a ray exceeded the traversal step cap */
#define TRACER_ERR_STACK_OVERFLOW (-8)      /* traversal stack too shallow for the BVH */
#define TRACER_ERR_CUDA (-9)
#define TRACER_ERR_NO_SCENE (-10)
#define TRACER_ERR_BAD_BVH (-11)            /* BVH failed validation */

/* ------------------------------------------------------------ std430 records */

/* CameraData, Include/Camera.h:5-12 / struct Camera, Tracer.comp:22-35 (64 B) */
typedef struct tracer_camera {
    float pos[3];
    float _pad0;
    float dir[3];
    float _pad1;
    float right[3];
    float _pad2;
    float up[3];
    float _pad3;
} tracer_camera;

/* FrameData push constants, Include/GraphicsDevice.h:20-29 /
 * Tracer.comp:151-166 (96 B).  light_pos is carried but unused (deprecated in
 * the shader, Tracer.comp:158-161). */
typedef struct tracer_frame {
    float aspect_ratio;
    float seed;
    float _pad0[2];
    float light_pos[3];
    float _pad1;
    tracer_camera camera;
} tracer_frame;

#define TRACER_MAT_DIFFUSE 0u    /* Tracer.comp:51 */
#define TRACER_MAT_DIELECTRIC 1u /* Tracer.comp:52; IOR read from roughness */

/* struct Material, Tracer.comp:59-74 (48 B: albedo@0 emissive@16
 * roughness@28 metalness@32 type@36) */
typedef struct tracer_material {
    float albedo[3];
    uint32_t _pad0;
    float emissive[3];
    float roughness;
    float metalness;
    uint32_t type;
    uint32_t _pad1[2];
} tracer_material;

/* struct Sphere, Tracer.comp:102-111 (64 B) */
typedef struct tracer_sphere {
    tracer_material mat;
    float P[3];
    float r;
} tracer_sphere;

/* struct Plane, Tracer.comp:118-125 (64 B) */
typedef struct tracer_plane {
    tracer_material mat;
    float N[3];
    float len;
} tracer_plane;

/* struct Triangle, Tracer.comp:127-132 / Include/GraphicsDevice.h:13-18
 * (48 B).  The reference gives every triangle the constant material `mirror`
 * (Tracer.comp:386); here v0's padding lane holds an index into the scene's
 * material table, so a table whose entry 0 is `mirror` reproduces it. */
typedef struct tracer_triangle {
    float v0[3];
    uint32_t material;
    float v1[3];
    uint32_t _pad1;
    float v2[3];
    uint32_t _pad2;
} tracer_triangle;

/* BVH node (32 B; the reference has no BVH).  count > 0: leaf holding
 * primitives prim_index[left_or_first .. left_or_first + count); count == 0:
 * interior node whose children are nodes left_or_first and left_or_first + 1.
 * Node 0 is the root. */
typedef struct tracer_bvh_node {
    float bmin[3];
    int32_t left_or_first;
    float bmax[3];
    int32_t count;
} tracer_bvh_node;

/* ------------------------------------------------------------ BVH building */
#define TRACER_BVH_NONE 0   /* linear scan, as Tracer.comp:378-428 */
#define TRACER_BVH_MEDIAN 1 /* median split on the longest centroid axis */
#define TRACER_BVH_SAH 2    /* binned surface-area heuristic */

#define TRACER_PRIM_TRIANGLE 0
#define TRACER_PRIM_SPHERE 1

/* Builds a BVH over n triangles (tracer_triangle) or spheres (tracer_sphere).
 * nodes_out needs room for 2n - 1 nodes, prim_index_out for n entries.
 * Node boxes are padded outward slightly so that floating-point rounding in
 * traversal never culls a box whose primitive a ray hits.  Deterministic:
 * the same input gives the same nodes on every host. */
int tracer_build_bvh(int kind, int prim_type, const void* prims, uint32_t n, uint32_t leaf_size, uint32_t sah_bins,
                     tracer_bvh_node* nodes_out, uint32_t* num_nodes_out, uint32_t* prim_index_out,
                     uint32_t* depth_out);

/* Checks a BVH: indices in range, every primitive referenced exactly once,
 * each box contains its children's boxes and its primitives.  Returns
 * TRACER_OK or TRACER_ERR_BAD_BVH; *depth_out gets the tree depth. */
int tracer_validate_bvh(int prim_type, const void* prims, uint32_t n, const tracer_bvh_node* nodes,
                        uint32_t num_nodes, const uint32_t* prim_index, uint32_t* depth_out);

/* ------------------------------------------------------------ scene */
typedef struct tracer_scene_desc {
    const tracer_triangle* triangles;
    uint32_t num_triangles;
    const tracer_material* materials; /* table indexed by tracer_triangle.material */
    uint32_t num_materials;
    const tracer_sphere* spheres;
    uint32_t num_spheres;
    const tracer_plane* planes; /* always scanned linearly (unbounded) */
    uint32_t num_planes;
    int32_t bvh;        /* TRACER_BVH_*; NONE = linear scan of triangles and spheres */
    uint32_t leaf_size; /* 0 = 2 (median) / 4 (SAH) */
    uint32_t sah_bins;  /* 0 = 16 */
    /* Optional prebuilt BVHs (validated on upload); NULL = build here. */
    const tracer_bvh_node* tri_nodes;
    uint32_t num_tri_nodes;
    const uint32_t* tri_prim_index;
    const tracer_bvh_node* sphere_nodes;
    uint32_t num_sphere_nodes;
    const uint32_t* sphere_prim_index;
} tracer_scene_desc;

/* ------------------------------------------------------------ tracing */
#define TRACER_TIES_REFERENCE 0 /* Tracer.comp:382/:402/:418 scan-order rule; linear scan only */
#define TRACER_TIES_STRICT 1    /* nearest (t, primitive id) below tmax; required with a BVH */

#define TRACER_KERNEL_AUTO 0      /* WAVEFRONT for BVH scenes with >= 2^16 pixel x spp x depth when the
                                     scene has an 8-wide BVH (and bvh_width is 0 or 8), >= 2^22 otherwise;
                                     else PLAIN (tracer_trace_adjoint: WAVEFRONT wherever it applies) */
#define TRACER_KERNEL_PLAIN 1     /* one thread per pixel, nested sample/bounce loops */
#define TRACER_KERNEL_WAVEFRONT 2 /* persistent extend kernel + shade kernel over path queues */

#define TRACER_AOV_RGBA8 0       /* w*h*4 u8: what imageStore writes (Tracer.comp:592) */
#define TRACER_AOV_RGBA32F 1     /* w*h*4 f32: the colour before UNORM8 conversion */
#define TRACER_AOV_PRIMARY_HIT 2 /* w*h*(u32 prim id, f32 t) of the first ray of each pixel */
#define TRACER_AOV_STATS 3       /* one tracer_stats */
#define TRACER_AOV_LINEAR 4      /* w*h*4 f32: mean radiance accum / spp before tone mapping, alpha 1 */

/* Primitive ids in PRIMARY_HIT: triangles 0..nt-1, spheres nt..nt+ns-1,
 * planes after; 0xFFFFFFFF (and t = -1) on a miss. */

typedef struct tracer_trace_params {
    uint32_t width, height; /* storage-image size (RAYTRACE_RESOLUTION^2 in the reference) */
    uint32_t spp;           /* SAMPLES, Tracer.comp:180 (reference 4) */
    uint32_t max_depth;     /* DEPTH, Tracer.comp:179 (reference 4) */
    uint32_t rr_start;      /* first depth with Russian roulette (reference 0: every depth) */
    float sky[3];           /* radiance returned by a miss (reference 0) */
    int32_t tie_mode;       /* TRACER_TIES_* */
    int32_t kernel;         /* TRACER_KERNEL_* */
    uint32_t block;         /* threads per block (multiple of 32, <= 1024); 0 = default */
    uint32_t stack_depth;   /* traversal stack entries per thread; 0 = BVH depth */
    uint32_t wavefront;     /* wavefront extend kernel: resident CTAs per SM; 0 = occupancy maximum */
    uint32_t aov_mask;      /* bit (1 << TRACER_AOV_*) per image written; 0 = RGBA8 only */
    uint32_t stats;         /* nonzero: count rays, node fetches and primitive tests */
    uint32_t bvh_width;     /* wavefront traversal: 0 = auto (= 2), 2 = the binary BVH, 4 = 4-wide nodes
                               collapsed from it (same boxes, same hits; measured slower on sparse
                               triangle soups, where it tests boxes the binary traversal culls) */
    uint32_t tail_paths;    /* wavefront: once fewer than this many paths are live, one kernel runs each of
                               them to the end of its pixel (remaining bounces and samples) instead of
                               further rounds; a frame with fewer pixels than this runs no round at all.
                               0 = auto: twice the extend kernel's resident threads, no round below once
                               that; 1 = never.  Same images either way. */
} tracer_trace_params;

typedef struct tracer_stats {
    uint64_t closest_rays; /* trace_ray calls for the path (Tracer.comp:445) */
    uint64_t shadow_rays;  /* trace_ray calls for next-event estimation (:473) */
    uint64_t node_fetches; /* 32 B BVH node records read */
    uint64_t tri_tests;    /* 48 B triangle records tested */
    uint64_t sphere_tests; /* 64 B sphere records tested */
    uint64_t plane_tests;  /* 64 B plane records tested */
    uint64_t hits;         /* closest-hit rays that found a hit (each reads a 48 B material) */
} tracer_stats;

typedef struct tracer_ctx tracer_ctx;

/* Replaces GraphicsDevice::Construct's compute set-up (GraphicsDevice.cpp:986-1131). */
int tracer_create(tracer_ctx** out, int cuda_device);
/* Replaces GraphicsDevice::Destruct for the tracer's resources. */
void tracer_destroy(tracer_ctx* ctx);
const char* tracer_last_error(const tracer_ctx* ctx);
const char* tracer_status_string(int status);
/* Bound for every wait on the GPU (default 60000 ms). */
int tracer_set_timeout(tracer_ctx* ctx, uint32_t timeout_ms);
/* Cap on the BVH traversal steps of one ray (no counterpart in the
 * reference, whose linear scan has no such loop).  0 = automatic: twice the
 * BVH's node count plus 16, which a valid BVH never reaches.  A ray that
 * reaches the cap ends its traversal with the best hit found so far, the
 * kernels run to completion, and the next wait reports
 * TRACER_ERR_TRAVERSAL_LIMIT; the context stays usable.  For exercising that
 * failure path; applies to every later trace of the context. */
int tracer_set_traversal_limit(tracer_ctx* ctx, uint32_t steps);

/* Replaces the scene SSBO upload (GraphicsDevice.cpp:796-822).  Copies the
 * arrays to the GPU, building or validating BVHs; replaces any previous scene. */
int tracer_upload_scene(tracer_ctx* ctx, const tracer_scene_desc* desc);

/* Replaces the material table of the current scene in place (same count). */
int tracer_set_materials(tracer_ctx* ctx, const tracer_material* materials, uint32_t num_materials);

/* Replaces vkCmdPushConstants + vkCmdDispatch (GraphicsDevice.cpp:1264-1266).
 * Asynchronous and ordered on cuda_stream (a cudaStream_t; NULL = the
 * context's own stream).  frame is copied by value, like a push constant. */
int tracer_trace(tracer_ctx* ctx, const tracer_frame* frame, const tracer_trace_params* params, void* cuda_stream);

/* Waits (bounded) for the last trace, reports device-side errors, and copies
 * one AOV to host memory; bytes must equal the AOV's size. */
int tracer_readback(tracer_ctx* ctx, int aov, void* host_dst, size_t bytes);

/* Waits (bounded) for the last trace and reports device-side errors. */
int tracer_synchronize(tracer_ctx* ctx);

/* Device address and size of an AOV of the last trace (zero-copy interop;
 * valid until the next trace with a different image size). */
int tracer_device_image(tracer_ctx* ctx, int aov, void** device_ptr, size_t* bytes);

/* ------------------------------------------------------------ adjoint
 * Gradients of an image loss L with respect to the material table's albedo
 * and emission and to the camera position (no counterpart in the reference).
 * dL_dimage: w*h*4 floats, dL/dI for the RGBA32F image of the same frame and
 * params (alpha ignored).  linear_image: the LINEAR AOV of the forward trace
 * of that frame (w*h*4 floats), or NULL to recompute it.  Outputs (any may be
 * NULL): d_albedo and d_emission num_materials*3 floats, d_campos 3 floats.
 * Each pointer may be host or device memory; with host outputs the call
 * waits (bounded) for the result, with device outputs it is asynchronous on
 * cuda_stream.  Path replay: every sample is traced again (pass 1, giving
 * its radiance) and then replayed with the gradient terms (pass 2, the same
 * rays, traced again: no path vertices are stored).  As an option
 * (tracer_set_adjoint_hit_log), the wavefront form (scenes without emissive
 * spheres) keeps pass 1's closest hits of each pixel's current sample (16
 * bytes x max_depth per pixel) and pass 2 reads them instead of tracing.
 * The Russian-roulette normalisation is treated as a constant.  Materials of spheres and planes (stored inline) get no gradient.
 * d_campos is the interior part (the camera position enters next-event
 * shading through the view vector and the hit points: the derivative of the
 * point-sampled image away from outlines, zero for scenes without emissive
 * spheres) plus, when tracer_set_edge_sampling has turned it on, the boundary
 * part: the image changes as triangle outlines move across pixels, which is
 * the derivative of each pixel averaged over a one-pixel box around its
 * sample point (edge sampling of primary visibility; outlines seen only by
 * bounce rays, and sphere outlines, are not included).  The boundary part
 * re-evaluates every pixel an outline crosses on both sides of it, which on
 * the 10k-triangle soup at 256^2 x 4 spp costs about as much as the rest of
 * the adjoint (1.0 against 0.86 ms). */
int tracer_trace_adjoint(tracer_ctx* ctx, const tracer_frame* frame, const tracer_trace_params* params,
                         const float* dL_dimage, const float* linear_image, float* d_albedo, float* d_emission,
                         float* d_campos, void* cuda_stream);

/* Turns on the boundary part of d_campos in tracer_trace_adjoint and sets
 * how many pieces each triangle edge's image is split into (one GPU thread
 * each; each piece is integrated exactly over the pixel boxes it crosses, so
 * this is a parallelism setting, 4 being a good value); 0 = off, the
 * default.  At most 1024.  Applies to every later adjoint of the context.
 * No counterpart in the reference. */
int tracer_set_edge_sampling(tracer_ctx* ctx, uint32_t samples_per_edge);

/* Device memory the wavefront adjoint may keep pass 1's closest hits in
 * (width x height x max_depth x 16 bytes; allocated on first use and kept
 * for later adjoints of the context): pass 2 then replays them without
 * tracing, which halves the adjoint's traced rays with the same gradients
 * (c3: 0.48 against 0.79 ms).  A trace whose hits would exceed the limit
 * traces pass 2 instead.  0 = never keep them, the default: pure path replay,
 * no stored path vertices (frees the buffer).  No counterpart in the
 * reference. */
int tracer_set_adjoint_hit_log(tracer_ctx* ctx, uint64_t max_bytes);

/* ------------------------------------------------------------ batches
 * Many independent scenes of uneven size and resolution traced together (no
 * counterpart in the reference, which renders one fixed scene).  The scenes'
 * triangles, BVHs, materials, spheres and planes are packed into one device
 * arena; all scenes' paths share the wavefront queues, so small scenes fill
 * the GPU together instead of one under-filled launch each. */

/* Uploads n scenes into the context's batch arena (replacing any previous
 * batch; the single-scene state of tracer_upload_scene is separate).  BVHs
 * are built per scene on host threads.  Batches need a BVH (bvh != NONE). */
int tracer_upload_scenes(tracer_ctx* ctx, const tracer_scene_desc* descs, uint32_t n);

/* Traces every scene of the batch: frames[i] and params[i] describe scene i
 * (image size, spp, depth, RR start, sky; strict ties).  kernel, block,
 * stack_depth, wavefront, aov_mask and stats are taken from params[0].
 *   kernel = WAVEFRONT: one wavefront over all scenes.  use_graph != 0 runs
 *     it as one CUDA graph (generate + every round, captured once per batch
 *     shape and replayed), so the host neither launches per round nor waits.
 *   kernel = PLAIN: the plain kernel launched once per scene, in order (the
 *     per-scene baseline).
 * Asynchronous on cuda_stream like tracer_trace. */
int tracer_trace_batched(tracer_ctx* ctx, const tracer_frame* frames, const tracer_trace_params* params, uint32_t n,
                         int use_graph, void* cuda_stream);

/* Like tracer_readback, for scene `scene` of the last batched trace. */
int tracer_readback_scene(tracer_ctx* ctx, uint32_t scene, int aov, void* host_dst, size_t bytes);

/* Per-kernel GPU time of the last trace, measured with CUDA events when
 * profiling is on (off by default; the reference has only an FPS counter,
 * Source/Main.cpp:152-163). */
typedef struct tracer_timings {
    float total_ms;     /* whole trace */
    float extend_ms;    /* wavefront: sum over rounds of the extend (traversal) kernel */
    float shade_ms;     /* wavefront: sum over rounds of the shade kernel */
    uint32_t rounds;    /* wavefront rounds (extend + shade) */
    uint32_t launches;  /* kernels launched */
    float finish_ms;    /* wavefront: the kernel that finished the last paths (tail_paths), 0 if none ran */
} tracer_timings;
int tracer_set_profiling(tracer_ctx* ctx, int enable);
int tracer_last_timings(tracer_ctx* ctx, tracer_timings* out);

/* Per-round detail of the last single-scene wavefront trace made with
 * profiling on: live paths at the start of each round and its kernel times.
 * When the finishing kernel ran, the last entry is its own (finish = 1, its
 * time in extend_ms).  Writes min(cap, entries) records, the count to *n. */
typedef struct tracer_round_info {
    uint32_t paths;   /* paths queued for the round */
    uint32_t finish;  /* 1: the finishing kernel */
    float extend_ms;
    float shade_ms;
} tracer_round_info;
int tracer_last_rounds(tracer_ctx* ctx, tracer_round_info* out, uint32_t cap, uint32_t* n);

/* Trace that allocates no memory during the call.  No counterpart in the
 * reference (its Vulkan device allocates all its buffers up front in
 * GraphicsDevice::Construct).
 *
 * For callers that must not allocate device memory while rendering: a frame
 * loop with a fixed time budget, where a cudaMalloc/cudaFree can synchronize
 * the whole device and stall the frame, or a host engine that owns every
 * device allocation through its own pool and hands libraries only buffers it
 * has already allocated.  Such a caller creates the context and uploads the
 * scene once at start-up, then calls this entry point per frame.
 *
 * It runs the wavefront kernels on the scene uploaded to ctx, 128 threads per
 * block, binary traversal (bvh_width 0 or 2; other widths are refused; the
 * block field is not read), with no queue length read back: when the image
 * has fewer pixels than tail_paths -- always with the automatic threshold,
 * which is the extend kernel's resident threads as in tracer_trace -- the
 * generate kernel and one finishing launch; otherwise (tail_paths = 1, or a
 * tail_paths at most the pixel count) every one of the spp * max_depth + 1
 * rounds is launched (2 kernels each, a round with no live path returning at
 * once).  It writes the
 * image straight into caller-owned device buffers: rgba8_out (w*h*4 bytes)
 * and/or rgba32f_out (w*h*16 bytes); either may be NULL, not both.  The
 * wavefront's path state, queues and counters live in one fixed array of
 * device memory inside the library (about 1.8 MB, reserved on every GPU that
 * loads the library until the process exits), so images are limited to
 * TRACER_NOALLOC_MAX_PIXELS pixels and spp * max_depth to
 * TRACER_NOALLOC_MAX_ROUNDS; larger requests return
 * TRACER_ERR_NO_SUITABLE_SURFACE / TRACER_ERR_INVALID_ARG with a message.
 * The first call on a device looks up that array's device address, so make
 * the first call on each device before any stream capture.  All calls share
 * the one array and each leaves its contents behind (the kernels clear what
 * must start at zero); calls that may overlap on the GPU -- on different
 * streams, or on several contexts of one device -- race on it and must be
 * ordered by the caller.  Asynchronous on cuda_stream (NULL = the context's
 * stream); the traversal status words are not read back (with a validated
 * BVH they cannot trip). */
#define TRACER_NOALLOC_MAX_PIXELS 16384u /* e.g. 128 x 128 */
#define TRACER_NOALLOC_MAX_ROUNDS 8192u  /* spp * max_depth */
int tracer_trace_noalloc(tracer_ctx* ctx, const tracer_frame* frame, const tracer_trace_params* params,
                         void* rgba8_out, void* rgba32f_out, void* cuda_stream);

/* ------------------------------------------------------------ present pass
 * The step after the dispatch: the reference's fragment shader
 * Assets/Fullscreen.frag, drawn over the window by a fullscreen triangle
 * (Assets/Fullscreen.vert) in GraphicsDevice::Draw (Source/
 * GraphicsDevice.cpp:1286-1308), here into a headless framebuffer.  Per
 * output pixel: the traced image is sampled at the pixel's uv, flipped
 * vertically (the traced image's row 0 is its bottom), with bilinear
 * filtering and clamp-to-border black (GraphicsDevice.cpp:770-790); where the
 * squared difference to the previous frame's image exceeds 0.0005 the
 * output is the mean of four taps half a texel of a 1024^2 image away (1/2048
 * in uv, Fullscreen.frag:12), else the centre tap.  The framebuffer's row 0
 * is its top row; channels are in RGBA order (the reference's swapchain is
 * B8G8R8A8_UNORM: the same bytes, swizzled). */
typedef struct tracer_present_params {
    uint32_t width, height; /* framebuffer extent (the reference's window, 1024 x 768, Main.cpp:92) */
    uint32_t out_aov;       /* TRACER_AOV_RGBA8 (UNORM8) or TRACER_AOV_RGBA32F */
    uint32_t mode;          /* tracer_draw: TRACER_PRESENT_PINGPONG or TRACER_PRESENT_ACCUMULATE */
} tracer_present_params;

/* Frame k is traced into image slot k % 2 and the present pass reads slot 0
 * as the current image and slot 1 as the previous one, as the reference binds
 * them (traced_images, Source/VulkanState.h:106-108, bound at
 * GraphicsDevice.cpp:955-983; currentFrame alternates, :1341). */
#define TRACER_PRESENT_PINGPONG 0u
/* Progressive accumulation (no counterpart in the reference): the frames'
 * linear radiance (LINEAR AOV) is summed on the device while the camera,
 * aspect ratio, trace parameters and scene stay the same (any change, or
 * tracer_draw_reset, restarts the sum); the present pass reads the
 * tonemapped mean after this frame as the current image and the mean before
 * it as the previous one, so its variance test sees the estimate converge.
 * Pass a new frame seed per call for new samples. */
#define TRACER_PRESENT_ACCUMULATE 1u

/* The present pass alone over caller images: image0 is the image bound as
 * raytraced_image, image1 as prev_raytraced_image; both src_width x
 * src_height, TRACER_AOV_RGBA8 (4 bytes per texel) or TRACER_AOV_RGBA32F (16
 * bytes), host or device memory.  out: width*height*4 bytes (RGBA8) or *16
 * (RGBA32F), host (the call waits, bounded) or device (asynchronous on
 * cuda_stream).  pp->mode is ignored. */
int tracer_present(tracer_ctx* ctx, const void* image0, const void* image1, uint32_t src_width, uint32_t src_height,
                   int src_aov, const tracer_present_params* pp, void* out, size_t out_bytes, void* cuda_stream);

/* One GraphicsDevice::Draw (GraphicsDevice.cpp:1236-1343) without the window:
 * tracer_trace of frame/params (RGBA8, plus LINEAR in ACCUMULATE mode, are
 * added to params->aov_mask), then the present pass into out as for
 * tracer_present.  The frame's seed and aspect ratio are used as given (the
 * reference sets them per frame: rand() / RAND_MAX and the swapchain's
 * aspect, GraphicsDevice.cpp:1258-1262). */
int tracer_draw(tracer_ctx* ctx, const tracer_frame* frame, const tracer_trace_params* params,
                const tracer_present_params* pp, void* out, size_t out_bytes, void* cuda_stream);

/* Clears both frame slots (to black) and the accumulation; the next draw is
 * frame 0. */
int tracer_draw_reset(tracer_ctx* ctx);

/* ------------------------------------------------------------ legacy Whitted shader
 * Assets/Raytracer.comp, the reference's second compute shader, which its
 * program does not load (it dispatches Tracer.comp): a Whitted ray tracer over
 * its own constant scene (one triangle, two spheres, five planes), one point
 * light at frame->light_pos with a shadow ray, two mirror bounces.  Reads
 * frame's aspect_ratio, light_pos and camera (the shader's push-constant
 * offsets equal FrameData's) and params' width, height, aov_mask (RGBA8,
 * RGBA32F, STATS) and stats; needs no uploaded scene.  Output as for
 * tracer_trace (tracer_readback). */
int tracer_trace_whitted(tracer_ctx* ctx, const tracer_frame* frame, const tracer_trace_params* params,
                         void* cuda_stream);

/* ------------------------------------------------------------ camera
 * The reference's camera controller (Camera, Source/Camera.cpp:5-64) with the
 * input handling of its main loop (Source/Main.cpp:23-83), for scripted
 * camera paths: a sequence of per-frame inputs gives the FrameData camera of
 * every frame.  Host only, single precision, no fused multiply-add. */
typedef struct tracer_camera_controller {
    tracer_camera data;   /* CameraData: pos, dir, right, up */
    float front[3];       /* CameraDataAux::front */
    float pitch, yaw;     /* degrees */
    float last_mouse[2];  /* last cursor position seen (Main.cpp:17-18) */
    uint32_t light_locked; /* light_pos follows the camera (Main.cpp:20, :178) */
    float light_pos[3];   /* FrameData::light_pos: (0, 64, 0) at start (Main.cpp:141) */
} tracer_camera_controller;

#define TRACER_KEY_W 1u  /* move_forward  (Main.cpp:27-30) */
#define TRACER_KEY_S 2u  /* move_backward, only without W */
#define TRACER_KEY_A 4u  /* move_left */
#define TRACER_KEY_D 8u  /* move_right, only without A */
#define TRACER_KEY_R 16u /* move_up */
#define TRACER_KEY_F 32u /* move_down, only without R */

/* One frame of input, applied in the order of the main loop (Main.cpp:150-180):
 * cursor events (mouse_callback) and the E key (key_callback) arrive while
 * events are polled, then the held keys move the camera by 111 * dt. */
typedef struct tracer_input_frame {
    float dt;               /* seconds since the previous frame */
    uint32_t keys;          /* TRACER_KEY_* held */
    uint32_t toggle_light;  /* E pressed this frame */
    uint32_t has_cursor;    /* a cursor event at (cursor_x, cursor_y) */
    double cursor_x, cursor_y;
} tracer_input_frame;

/* Camera::Camera(): pos (0, 64, -48), pitch 0, yaw 90 (Camera.cpp:5-10). */
void tracer_camera_init(tracer_camera_controller* cam);
/* The start-up camera of the reference's main loop (Main.cpp:134-139). */
void tracer_camera_init_startup(tracer_camera_controller* cam);
/* Camera::update (Camera.cpp:48-64): pitch clamped to [-89, 89]; front from
 * pitch and yaw; dir, right, up from front. */
void tracer_camera_update(tracer_camera_controller* cam);
/* Camera::move_forward .. move_down (Camera.cpp:12-46), direction 0..5 =
 * forward, backward, left, right, up, down. */
int tracer_camera_move(tracer_camera_controller* cam, int direction, float speed);
/* mouse_callback (Main.cpp:66-83) for a cursor event at (x, y). */
void tracer_camera_cursor(tracer_camera_controller* cam, double x, double y);
/* poll_keyboard (Main.cpp:23-51). */
void tracer_camera_keys(tracer_camera_controller* cam, uint32_t keys, float dt);
/* Applies n frames of input; frames_out[i] (may be NULL) receives the frame's
 * FrameData camera and light_pos (which follows the camera position +
 * (0, -1, 0) while the light is locked and stays put otherwise, Main.cpp:
 * 176-178); aspect_ratio and seed are left as they were in frames_out[i]. */
int tracer_camera_script(tracer_camera_controller* cam, const tracer_input_frame* inputs, uint32_t n,
                         tracer_frame* frames_out);

/* ------------------------------------------------------------ measurement
 * No counterpart in the reference.  Read bandwidth of an L2-resident buffer of
 * `bytes` (read `passes` times per launch with loads that bypass L1), in GB/s
 * of bytes delivered: the denominator for kernels whose working set lives in
 * L2.  Allocates and frees its buffer; synchronous. */
int tracer_measure_l2_read(tracer_ctx* ctx, size_t bytes, uint32_t passes, double* gbs);

#ifdef __cplusplus
}
#endif

#endif /* TRACER_ABI_H */
