/* C interface of the CPU oracle (test infrastructure; see tracer_oracle.cpp).
 * Scene arrays use the same std430 records as the product's C ABI. */
#ifndef ORACLE_API_H
#define ORACLE_API_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_scene {
    const float* triangles;       /* 48 B records; v0.w lane = material id (u32) */
    uint32_t num_triangles;
    const float* materials;       /* 48 B records */
    uint32_t num_materials;
    const float* spheres;         /* 64 B records (Material + centre + radius) */
    uint32_t num_spheres;
    const float* planes;          /* 64 B records (Material + normal + offset) */
    uint32_t num_planes;
    const void* tri_nodes;        /* 32 B BVH nodes over triangles, or NULL = linear scan */
    uint32_t num_tri_nodes;
    const uint32_t* tri_prim_index;
    const void* sphere_nodes;     /* 32 B BVH nodes over spheres, or NULL */
    uint32_t num_sphere_nodes;
    const uint32_t* sphere_prim_index;
} oracle_scene;

typedef struct oracle_params {
    uint32_t width, height, spp, max_depth, rr_start;
    float sky[3];
    int32_t tie_mode;   /* 0 = reference ties (linear scan), 1 = strict */
    int32_t trig_mode;  /* 0 = portable cos/sin (rng_trig.h), 1 = libm */
    int32_t threads;    /* 0 = all OpenMP threads */
    uint32_t row_begin, row_end, row_step;  /* scanline subset; row_end 0 = height */
} oracle_params;

typedef struct oracle_stats {
    uint64_t closest_rays, shadow_rays, node_fetches, tri_tests, sphere_tests, plane_tests, hits;
} oracle_stats;

int oracle_render(const oracle_scene* scene, const float* frame96, const oracle_params* params, float* rgba32f,
                  uint8_t* rgba8, uint32_t* hit_id, float* hit_t, oracle_stats* stats);
/* FP64 evaluation (the RNG stays float).  accum: 4 doubles per pixel = the
 * mean radiance accum / spp (3) and the pixel's dither rand() / 64. */
int oracle_render_f64(const oracle_scene* scene, const float* frame96, const oracle_params* params, float* rgba32f,
                      double* accum, oracle_stats* stats);
void oracle_rand(float cx, float cy, float salt, int trig_mode, int n, float* out);
float oracle_cos(float x);
float oracle_sin(float x);
float oracle_tri_intersect(const float* o, const float* d, const float* tri48);
float oracle_sphere_intersect(const float* o, const float* d, const float* c, float radius);
float oracle_plane_intersect(const float* o, const float* d, const float* n, float len);
int oracle_trace_ray(const oracle_scene* scene, int tie_mode, int shadow, const float* o, const float* d, float tmax,
                     float* out, oracle_stats* stats);
void oracle_radiance(const oracle_scene* scene, const float* frame96, const oracle_params* params, const float* o,
                     const float* d, float cx, float cy, float salt, float* out_rgb, float* out_salt);

/* present_oracle.cpp: the present pass (Fullscreen.frag), progressive
 * accumulation and the camera controller (Camera.cpp, Main.cpp input). */
void oracle_present(const void* image0, const void* image1, int src_is_float, uint32_t src_w, uint32_t src_h,
                    uint32_t width, uint32_t height, float* out_rgba32f, uint8_t* out_rgba8);
void oracle_accumulate(const float* linear_rgba, float* sum_rgba, uint32_t n_pixels, uint32_t n,
                       float* display_rgba);

/* whitted_oracle.cpp: the legacy Whitted shader (Assets/Raytracer.comp) over
 * its constant scene; frame: the 96-byte FrameData. */
void oracle_whitted(const float* frame96, uint32_t width, uint32_t height, float* rgba32f, uint8_t* rgba8,
                    oracle_stats* stats);

/* bvh_oracle.cpp: the oracle's own BVH builder (kind 1 = median split, 2 =
 * binned SAH; prim_type 0 = 48 B triangles, 1 = 64 B spheres), node for node
 * the product's definition (32 B nodes, children side by side, root 0).
 * nodes_out: room for 2n - 1 nodes.  Returns 0, or -1 on bad arguments. */
int oracle_build_bvh(int kind, int prim_type, const void* prims, uint32_t n, uint32_t leaf_size, uint32_t bins,
                     void* nodes_out, uint32_t* num_nodes, uint32_t* prim_index_out, uint32_t* depth_out);

typedef struct oracle_camera_ctl {
    float cam[16];        /* CameraData: pos, dir, right, up (16-byte lanes) */
    float front[3];
    float pitch, yaw;     /* degrees */
    float last_mouse[2];
} oracle_camera_ctl;
void oracle_camera_init(oracle_camera_ctl* c);
void oracle_camera_update(oracle_camera_ctl* c);
void oracle_camera_move(oracle_camera_ctl* c, int dir, float speed);
void oracle_camera_mouse(oracle_camera_ctl* c, double x, double y);
void oracle_camera_keyboard(oracle_camera_ctl* c, uint32_t keys, float dt);

#ifdef __cplusplus
}
#endif

#endif
