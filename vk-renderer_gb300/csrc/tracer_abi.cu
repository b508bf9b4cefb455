// Host side of the C ABI (include/tracer_abi.h): context, scene upload,
// trace launch, bounded waits and readback.
//
// Replaces the compute portion of GraphicsDevice (Source/GraphicsDevice.cpp):
// scene SSBO creation and upload (:796-822), compute pipeline with the
// 96-byte push-constant range (:1089-1131), and the per-frame bind, push and
// dispatch (:1254-1266).  Where the reference ignores most Vulkan results and
// waits on fences forever (:1217), every call here returns a status and every
// wait on the GPU is bounded.

#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <algorithm>
#include <cmath>
#include <atomic>
#include <mutex>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "tracer_abi.h"
#include "tracer_core.cuh"
#include "tracer_edges.h"
#include "tracer_launch.h"
#include "tracer_present.h"
#include "bvh_cw8.h"
#include "bvh_wide.h"

using namespace vkt;

namespace {

template <class T> struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
};

struct SceneBuffers {
    DevBuf<float4> tri, mats, sph_geo, sph_rec, planes, tri_nodes, sph_nodes;
    DevBuf<float4> tri_wide, sph_wide;  // the BVHs as 4-wide nodes
    DevBuf<float4> tri_enc, sph_enc;    // the binary BVHs with pre-encoded child references
    DevBuf<float4> tri_cw8, tri_cw8_prims;  // compressed 8-wide BVH over the triangles, triangles in its order
    DevBuf<uint32_t> sph_id, emit;
    uint32_t nt = 0, nm = 0, ns = 0, np = 0, ne = 0;
    uint32_t n_tri_nodes = 0, n_sph_nodes = 0;
    uint32_t depth = 0;       // deepest BVH
    uint32_t wide_depth = 0;  // deepest 4-wide BVH
    bool wide = false;        // 4-wide nodes present
    uint32_t cw8_depth = 0;   // levels of the 8-wide BVH
    bool cw8 = false;         // 8-wide BVH present (triangle-only scenes)
    bool bvh = false;
    bool loaded = false;
    void release()
    {
        tri_wide.release();
        sph_wide.release();
        tri_enc.release();
        sph_enc.release();
        tri_cw8.release();
        tri_cw8_prims.release();
        tri.release();
        mats.release();
        sph_geo.release();
        sph_rec.release();
        planes.release();
        tri_nodes.release();
        sph_nodes.release();
        sph_id.release();
        emit.release();
        *this = SceneBuffers();
    }
};

struct AdjBuffers {
    DevBuf<float4> dldi, lin;
    DevBuf<double> grad;  // FP64 sums the kernel accumulates into
    DevBuf<float> gradf;  // the same, rounded to float for the outputs
    DevBuf<float4> pix;   // wavefront form: per-pixel delta and sample-start RNG state
    DevBuf<uint4> log;    // wavefront form: pass 1's closest hits of the current sample, per pixel
    DevBuf<float4> segs;  // boundary term: the visible outline parts the edge walk hands over
    DevBuf<uint32_t> nsegs;
    void release()
    {
        segs.release();
        nsegs.release();
        log.release();
        pix.release();
        dldi.release();
        lin.release();
        grad.release();
        gradf.release();
    }
};

}  // namespace

struct tracer_ctx {
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    bool pending = false;
    uint32_t timeout_ms = 60000;
    std::string err;
    SceneBuffers scene;
    // frame outputs
    uint32_t width = 0, height = 0;
    DevBuf<uchar4> rgba8;
    DevBuf<float4> rgba32f;
    DevBuf<uint2> hit;
    DevBuf<float4> linear;
    DevBuf<unsigned long long> stats;
    DevBuf<int> status;
    uint32_t last_mask = 0;
    // wavefront path state (scratch, one slot per pixel)
    DevBuf<float4> wf_ray_o, wf_ray_d, wf_acc, wf_mask, wf_accum;
    DevBuf<uint4> wf_hit;
    DevBuf<uint32_t> wf_prim0, wf_q0, wf_q1, wf_count, wf_scene;
    uint32_t* pinned_counts = nullptr;  // lagged queue lengths read by the launch loop
    std::vector<cudaEvent_t> count_events;
    // optional per-kernel timing of the last trace
    bool profiling = false;
    std::vector<cudaEvent_t> prof_events;  // 3 per round: before extend, after extend, after shade
    cudaEvent_t prof_begin = nullptr, prof_end = nullptr;
    uint32_t last_rounds = 0, last_launches = 0;
    uint32_t last_prof_rounds = 0;  // rounds of the last trace with per-kernel events recorded
    DevBuf<uint32_t> round_paths;   // profiling: live paths at the start of each round (+ the finish)
    uint32_t last_round_entries = 0;
    bool last_finish = false;       // the finishing kernel ran in the last trace
    uint32_t last_handover = 0;     // rounds before the finishing kernel in the last trace (if last_finish)
    int last_kernel = 0;
    // batch of scenes (tracer_upload_scenes / tracer_trace_batched)
    SceneBuffers batch;                 // arena: every scene's arrays back to back
    std::vector<DevScene> batch_scenes; // pointers into the arena, one per scene
    std::vector<uint32_t> batch_depth, batch_nodes;
    bool batch_emitters = false;
    DevBuf<TraceArgs> batch_slots;
    TraceArgs* pinned_slots = nullptr;
    uint32_t pinned_slots_n = 0;
    std::vector<size_t> batch_base;
    std::vector<uint32_t> batch_w, batch_h;
    DevBuf<uchar4> b_rgba8;
    DevBuf<float4> b_rgba32f;
    DevBuf<uint2> b_hit;
    uint32_t b_mask = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    std::vector<uint64_t> graph_key;
    uint64_t graph_rounds = 0;  // rounds in the graph, then the finishing kernel if graph_finish
    bool graph_finish = false;
    AdjBuffers adj;  // adjoint: dL/dI, linear image and gradient buffers
    // present pass and draw loop
    uint64_t scene_version = 0;       // bumped by every scene or material upload
    DevBuf<uchar4> slot[2];           // frame image slots (the reference's traced_images)
    uint32_t slot_w = 0, slot_h = 0;
    uint64_t draw_frame = 0;          // frames drawn since the last reset
    DevBuf<float4> acc_sum, acc_disp[2];
    uint32_t acc_n = 0;               // frames in acc_sum
    tracer_frame acc_frame;           // what the accumulated frames share
    tracer_trace_params acc_params;
    uint64_t acc_version = 0;
    DevBuf<unsigned char> pres_src[2], pres_out;  // staging for host images
    uint32_t trav_cap = 0;            // tracer_set_traversal_limit: 0 = automatic
    uint32_t edge_samples = 0;        // tracer_set_edge_sampling: pieces per triangle edge, 0 = off
    uint64_t adj_log_limit = 0;       // tracer_set_adjoint_hit_log: bytes for pass 1's hits, 0 = none (pure replay)
};

namespace {

int fail(tracer_ctx* c, int code, const char* fmt, ...)
{
    if (c) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        c->err = buf;
    }
    return code;
}

int cuda_fail(tracer_ctx* c, cudaError_t e, const char* what)
{
    if (e == cudaErrorMemoryAllocation) return fail(c, TRACER_ERR_OOM, "%s: out of device memory", what);
    return fail(c, TRACER_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

template <class T> cudaError_t dalloc(DevBuf<T>& b, size_t n)
{
    if (b.n == n && b.p) return cudaSuccess;
    b.release();
    if (n == 0) return cudaSuccess;
    cudaError_t e = cudaMalloc(&b.p, n * sizeof(T));
    if (e == cudaSuccess) b.n = n;
    return e;
}

template <class T> cudaError_t upload(DevBuf<T>& b, const T* src, size_t n)
{
    cudaError_t e = dalloc(b, n);
    if (e != cudaSuccess || n == 0) return e;
    return cudaMemcpy(b.p, src, n * sizeof(T), cudaMemcpyHostToDevice);
}

// Bounded wait on an event: polls instead of blocking so a stuck GPU turns
// into TRACER_ERR_TIMEOUT rather than a hang.
int wait_event(tracer_ctx* c, cudaEvent_t ev)
{
    auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        cudaError_t e = cudaEventQuery(ev);
        if (e == cudaSuccess) return TRACER_OK;
        if (e != cudaErrorNotReady) return cuda_fail(c, e, "waiting for the GPU");
        auto ms = std::chrono::duration_cast<std::chrono::milliseconds>(std::chrono::steady_clock::now() - t0).count();
        if (ms > (long long)c->timeout_ms)
            return fail(c, TRACER_ERR_TIMEOUT, "GPU did not finish within %u ms", c->timeout_ms);
        std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
}

int finish(tracer_ctx* c)
{
    if (!c->pending) return TRACER_OK;
    int r = wait_event(c, c->done);
    if (r != TRACER_OK) return r;
    c->pending = false;
    int st = 0;
    cudaError_t e = cudaMemcpy(&st, c->status.p, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(c, e, "reading the device status");
    if (st == ST_TRAVERSAL_LIMIT)
        return fail(c, TRACER_ERR_TRAVERSAL_LIMIT, "a ray exceeded the BVH traversal step limit");
    if (st == ST_STACK_OVERFLOW)
        return fail(c, TRACER_ERR_STACK_OVERFLOW, "traversal stack depth too small for the BVH");
    return TRACER_OK;
}

constexpr int kCountSlots = 8;  // ring of lagged queue-length copies
constexpr int kCountLag = 3;    // rounds the launch loop runs ahead of the GPU

void release_wavefront(tracer_ctx* c)
{
    c->wf_ray_o.release();
    c->wf_ray_d.release();
    c->wf_acc.release();
    c->wf_mask.release();
    c->wf_accum.release();
    c->wf_hit.release();
    c->wf_prim0.release();
    c->wf_q0.release();
    c->wf_q1.release();
    c->wf_scene.release();
}

cudaError_t ensure_wavefront(tracer_ctx* c, size_t npx)
{
    cudaError_t e = dalloc(c->wf_ray_o, npx);
    if (e == cudaSuccess) e = dalloc(c->wf_ray_d, npx);
    if (e == cudaSuccess) e = dalloc(c->wf_acc, npx);
    if (e == cudaSuccess) e = dalloc(c->wf_mask, npx);
    if (e == cudaSuccess) e = dalloc(c->wf_accum, npx);
    if (e == cudaSuccess) e = dalloc(c->wf_hit, npx);
    if (e == cudaSuccess) e = dalloc(c->wf_prim0, npx);
    if (e == cudaSuccess) e = dalloc(c->wf_q0, npx);
    if (e == cudaSuccess) e = dalloc(c->wf_q1, npx);
    if (e != cudaSuccess) release_wavefront(c);
    return e;
}

cudaEvent_t prof_event(tracer_ctx* c, size_t i)
{
    while (c->prof_events.size() <= i) {
        cudaEvent_t ev = nullptr;
        if (cudaEventCreate(&ev) != cudaSuccess) return nullptr;
        c->prof_events.push_back(ev);
    }
    return c->prof_events[i];
}

// Launches the wavefront: generate, then rounds of extend + shade until the
// path queue is empty (read back a few rounds behind the launches) or
// max_rounds is reached (no path needs more than spp * max_depth rounds).
// Once a read-back count is below tail, the finishing kernel runs the paths
// still queued to the end of their pixels and the rounds stop (counts never
// grow from round to round, so the lagged count bounds the current one).
// tail: 0 = twice the extend kernel's resident threads (below about one path
// per lane a round costs the latency of its slowest ray, whatever its size;
// measured on c1 with the finishing kernel as built: 1x 89.1 ms, 1.5x 88.6,
// 2x 88.5), 1 = never.  With fewer path slots than that from the start (for
// auto: fewer than the resident threads themselves), no round runs: the
// finishing kernel traces every pixel after generate (c3's 256^2 adjoint:
// 1.33 ms with four rounds first; a 640x360 frame of c1's scene, 230k
// pixels: 5.0 ms without rounds against 4.5 with them).
// With adj, the adjoint's generate, shade and finishing stages run instead of
// the forward's (a.linear = the forward image).
int run_wavefront(tracer_ctx* c, const TraceArgs& a, WfConfig& wc, size_t nslots, uint64_t max_rounds,
                  uint32_t stack, uint32_t wavefront, uint32_t tail, cudaStream_t st, const AdjWf* adj = nullptr)
{
    WfState ws{c->wf_ray_o.p, c->wf_ray_d.p, c->wf_hit.p, c->wf_acc.p, c->wf_mask.p, c->wf_accum.p,
               c->wf_prim0.p, {c->wf_q0.p, c->wf_q1.p}, c->wf_count.p, c->wf_scene.p};
    int per = wf_extend_blocks_per_sm(wc, stack);
    if (per <= 0) return fail(c, TRACER_ERR_INVALID_ARG, "extend kernel cannot be resident (stack %u)", stack);
    if (wavefront && (int)wavefront < per) per = (int)wavefront;
    wc.extend_grid = (uint32_t)(per * c->sm_count);
    const size_t sg = (nslots + 255) / 256;
    wc.shade_grid = (uint32_t)(sg < (size_t)c->sm_count * 8 ? sg : (size_t)c->sm_count * 8);
    const uint32_t resident = wc.extend_grid * wc.block;
    const uint32_t no_rounds_below = tail == 0 ? resident : tail;
    if (tail == 0) tail = 2 * resident;
    const int fin_per = tail <= 1 ? 0 : adj ? wf_adj_finish_blocks_per_sm(a, wc) : wf_finish_blocks_per_sm(wc, stack);
    if (fin_per <= 0) tail = 0;
    cudaError_t e = cudaSuccess;
    if (c->profiling) {
        e = dalloc(c->round_paths, (size_t)max_rounds + 1);
        if (e != cudaSuccess) return cuda_fail(c, e, "round statistics");
    }
    c->last_round_entries = 0;
    c->last_finish = false;
    c->last_handover = 0;
    if (adj) {
        e = cudaMemsetAsync(c->wf_count.p, 0, 3 * sizeof(uint32_t), st);
        if (e == cudaSuccess) e = wf_launch_adj_generate(a, ws, *adj, st);
    } else {
        e = wf_launch_generate(a, ws, wc, st);
    }
    c->last_launches += 1;
    if (e == cudaSuccess && tail > 1 && nslots < no_rounds_below) {
        const uint64_t blocks = ((uint64_t)nslots + 127) / 128;
        const uint64_t cap = (uint64_t)fin_per * c->sm_count;
        wc.finish_grid = (uint32_t)(blocks < cap ? blocks : cap);
        if (c->profiling) {
            cudaMemcpyAsync(c->round_paths.p, c->wf_count.p, sizeof(uint32_t), cudaMemcpyDeviceToDevice, st);
            c->last_round_entries = 1;
            cudaEventRecord(prof_event(c, 0), st);
        }
        e = adj ? wf_launch_adj_finish(a, ws, *adj, wc, 0, st) : wf_launch_finish(a, ws, wc, 0, st);
        if (c->profiling) cudaEventRecord(prof_event(c, 1), st);
        c->last_launches += 1;
        c->last_finish = true;
        c->last_handover = 0;
        c->last_rounds = 0;
        if (e != cudaSuccess) return cuda_fail(c, e, "wavefront launch");
        return TRACER_OK;
    }
    for (uint64_t r = 0; r < max_rounds && e == cudaSuccess; ++r) {
        const int qsel = (int)(r & 1);
        if (c->profiling) {
            cudaMemcpyAsync(c->round_paths.p + r, c->wf_count.p + qsel, sizeof(uint32_t), cudaMemcpyDeviceToDevice, st);
            c->last_round_entries = (uint32_t)(r + 1);
            cudaEventRecord(prof_event(c, 3 * r), st);
        }
        e = wf_launch_extend(a, ws, wc, qsel, st);
        if (c->profiling) cudaEventRecord(prof_event(c, 3 * r + 1), st);
        if (e == cudaSuccess) e = adj ? wf_launch_adj_shade(a, ws, *adj, wc, qsel, st) : wf_launch_shade(a, ws, wc, qsel, st);
        if (c->profiling) cudaEventRecord(prof_event(c, 3 * r + 2), st);
        c->last_launches += 2;
        c->last_rounds = (uint32_t)(r + 1);
        if (c->profiling && c->prof_events.size() >= 3 * (r + 1)) c->last_prof_rounds = (uint32_t)(r + 1);
        const int slot = (int)(r % kCountSlots);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(c->pinned_counts + slot, c->wf_count.p + (qsel ^ 1), sizeof(uint32_t),
                                cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaEventRecord(c->count_events[slot], st);
        if (e == cudaSuccess && r >= (uint64_t)kCountLag) {
            const int old = (int)((r - kCountLag) % kCountSlots);
            int w = wait_event(c, c->count_events[old]);
            if (w != TRACER_OK) return w;
            const uint32_t live = c->pinned_counts[old];
            if (live == 0) break;
            if (live < tail && r + 1 < max_rounds) {
                const uint64_t f = r + 1;
                const int fq = (int)(f & 1);
                const uint64_t blocks = ((uint64_t)live + 127) / 128;
                const uint64_t cap = (uint64_t)fin_per * c->sm_count;
                wc.finish_grid = (uint32_t)(blocks < cap ? blocks : cap);
                if (c->profiling) {
                    cudaMemcpyAsync(c->round_paths.p + f, c->wf_count.p + fq, sizeof(uint32_t),
                                    cudaMemcpyDeviceToDevice, st);
                    c->last_round_entries = (uint32_t)(f + 1);
                    cudaEventRecord(prof_event(c, 3 * f), st);
                }
                e = adj ? wf_launch_adj_finish(a, ws, *adj, wc, fq, st) : wf_launch_finish(a, ws, wc, fq, st);
                if (c->profiling) cudaEventRecord(prof_event(c, 3 * f + 1), st);
                c->last_launches += 1;
                c->last_finish = true;
                c->last_handover = (uint32_t)f;
                break;
            }
        }
    }
    if (e != cudaSuccess) return cuda_fail(c, e, "wavefront launch");
    return TRACER_OK;
}

// Traversal width of the wavefront's extend kernel.  bvh_width 8 (and auto,
// wherever the scene has it: triangle-only scenes) = the compressed 8-wide
// BVH, which needs no more stack than the binary traversal (at most one node
// group per 8-wide level); 2 = binary; 4 = the uncompressed 4-wide collapse,
// measured 8 % slower than binary on the soup workloads (visiting a collapsed
// node tests all four grandchildren's boxes where the binary traversal first
// culls with the parent's box, and most rays miss most boxes there); it
// pushes up to three children per level, so it needs 3 x (its depth) entries.
// stack: in, the binary traversal's stack; out, the stack of the chosen width
// (the shade and finishing kernels' binary traversals share it).
int pick_width_for(tracer_ctx* c, const tracer_trace_params* p, bool have_wide, uint32_t wide_depth, bool have_cw8,
                   uint32_t cw8_depth, uint32_t& stack, int& wide)
{
    wide = WF_WIDTH_2;
    if (p->bvh_width != 0 && p->bvh_width != 2 && p->bvh_width != 4 && p->bvh_width != 8)
        return fail(c, TRACER_ERR_INVALID_ARG, "bvh_width %u must be 0, 2, 4 or 8", p->bvh_width);
    if (p->bvh_width == 8 || (p->bvh_width == 0 && have_cw8)) {
        if (!have_cw8) return fail(c, TRACER_ERR_INVALID_ARG, "the scene has no 8-wide BVH (triangle-only scenes)");
        if (stack < cw8_depth) {
            if (p->stack_depth)
                return fail(c, TRACER_ERR_STACK_OVERFLOW, "8-wide traversal needs a stack of %u entries", cw8_depth);
            stack = cw8_depth;
        }
        wide = WF_WIDTH_8;
        return TRACER_OK;
    }
    if (!have_wide || p->bvh_width != 4) {
        if (p->bvh_width == 4) return fail(c, TRACER_ERR_INVALID_ARG, "the scene has no 4-wide BVH");
        return TRACER_OK;
    }
    const uint32_t need = 3 * wide_depth;
    const uint32_t ws = p->stack_depth ? p->stack_depth : need;
    if (ws < need || (size_t)ws * 256 * 8 > 200 * 1024) {
        if (p->bvh_width == 4)
            return fail(c, TRACER_ERR_STACK_OVERFLOW, "4-wide traversal needs a stack of %u entries", need);
        return TRACER_OK;
    }
    stack = ws;
    wide = WF_WIDTH_4;
    return TRACER_OK;
}

// Traversal steps a ray may take over a BVH of `nodes` nodes: each node is
// entered at most once per pass, so twice the node count (plus slack) is
// never reached by a valid BVH; tracer_set_traversal_limit overrides it.
uint32_t trav_limit(const tracer_ctx* c, uint32_t nodes)
{
    return c->trav_cap ? c->trav_cap : 2 * nodes + 16;
}

// Inverse of the matrix with columns dir, right, up (row-major), for the
// image projection of the camera's boundary term; false if singular.
bool camera_inverse(const tracer_camera& cam, float out[9])
{
    const double m[3][3] = {{cam.dir[0], cam.right[0], cam.up[0]},
                            {cam.dir[1], cam.right[1], cam.up[1]},
                            {cam.dir[2], cam.right[2], cam.up[2]}};
    const double det = m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) -
                       m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
                       m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
    if (!(std::fabs(det) > 1e-12)) return false;
    for (int r = 0; r < 3; ++r)
        for (int k = 0; k < 3; ++k) {
            // cofactor of (k, r) / det
            const int r0 = (k + 1) % 3, r1 = (k + 2) % 3, c0 = (r + 1) % 3, c1 = (r + 2) % 3;
            out[3 * r + k] = (float)((m[r0][c0] * m[r1][c1] - m[r0][c1] * m[r1][c0]) / det);
        }
    return true;
}

int pick_width(tracer_ctx* c, const tracer_trace_params* p, uint32_t& stack, int& wide)
{
    const SceneBuffers& s = c->scene;
    return pick_width_for(c, p, s.bvh && s.wide, s.wide_depth, s.bvh && s.cw8, s.cw8_depth, stack, wide);
}

// The 8-wide BVH of a triangle BVH and the triangles in its order: 64-byte
// records (v0, original id) (v1 - v0, leaf-ordered slot) (v2 - v0, 0) (0),
// from the leaf-ordered triangle records `tri` (3 float4 each, as uploaded).
// Returns false when the scene gets none (bvh_cw8.h).
bool make_cw8(const std::vector<tracer_bvh_node>& tnodes, const std::vector<float4>& tri, std::vector<Cw8Node>& nodes,
              std::vector<float4>& prims, uint32_t& depth)
{
    std::vector<uint32_t> order;
    if (tnodes.empty() || !build_cw8(tnodes.data(), (uint32_t)tnodes.size(), nodes, order, &depth)) return false;
    prims.assign(4 * order.size(), make_float4(0.0f, 0.0f, 0.0f, 0.0f));
    for (size_t k = 0; k < order.size(); ++k) {
        const uint32_t slot = order[k];
        const float4 a = tri[3 * (size_t)slot], b = tri[3 * (size_t)slot + 1], e = tri[3 * (size_t)slot + 2];
        float fslot;
        std::memcpy(&fslot, &slot, 4);
        prims[4 * k + 0] = make_float4(a.x, a.y, a.z, b.w);  // v0, original id
        prims[4 * k + 1] = make_float4(b.x, b.y, b.z, fslot);
        prims[4 * k + 2] = make_float4(e.x, e.y, e.z, 0.0f);
    }
    return true;
}

// Builds (or validates) one BVH; returns the leaf-order permutation.
int prepare_bvh(tracer_ctx* c, int kind, int prim_type, const void* prims, uint32_t n, uint32_t leaf, uint32_t bins,
                const tracer_bvh_node* given, uint32_t n_given, const uint32_t* given_idx,
                std::vector<tracer_bvh_node>& nodes, std::vector<uint32_t>& idx, uint32_t& depth)
{
    if (given) {
        if (!given_idx) return fail(c, TRACER_ERR_INVALID_ARG, "prebuilt BVH without a primitive index array");
        int r = tracer_validate_bvh(prim_type, prims, n, given, n_given, given_idx, &depth);
        if (r != TRACER_OK) return fail(c, TRACER_ERR_BAD_BVH, "prebuilt BVH failed validation");
        nodes.assign(given, given + n_given);
        idx.assign(given_idx, given_idx + n);
        return TRACER_OK;
    }
    nodes.resize(2 * (size_t)n);
    idx.resize(n);
    uint32_t nn = 0;
    int r = tracer_build_bvh(kind, prim_type, prims, n, leaf, bins, nodes.data(), &nn, idx.data(), &depth);
    if (r != TRACER_OK) return fail(c, r, "BVH build failed");
    nodes.resize(nn);
    return TRACER_OK;
}

}  // namespace

extern "C" {

const char* tracer_status_string(int s)
{
    switch (s) {
    case TRACER_OK: return "ok";
    case TRACER_ERR_NO_SUITABLE_GPU: return "no suitable GPU";
    case TRACER_ERR_NO_SUITABLE_SURFACE: return "no suitable surface";
    case TRACER_ERR_UNKNOWN: return "unknown error";
    case TRACER_ERR_INVALID_ARG: return "invalid argument";
    case TRACER_ERR_OOM: return "out of memory";
    case TRACER_ERR_TIMEOUT: return "timeout";
    case TRACER_ERR_TRAVERSAL_LIMIT: return "traversal step limit exceeded";
    case TRACER_ERR_STACK_OVERFLOW: return "traversal stack overflow";
    case TRACER_ERR_CUDA: return "CUDA error";
    case TRACER_ERR_NO_SCENE: return "no scene uploaded";
    case TRACER_ERR_BAD_BVH: return "invalid BVH";
    default: return "unrecognised status";
    }
}

int tracer_create(tracer_ctx** out, int cuda_device)
{
    if (!out) return TRACER_ERR_INVALID_ARG;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return TRACER_ERR_NO_SUITABLE_GPU;
    if (cuda_device < 0 || cuda_device >= n) return TRACER_ERR_NO_SUITABLE_GPU;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, cuda_device) != cudaSuccess) return TRACER_ERR_NO_SUITABLE_GPU;
    // The kernels are built for sm_103a only.
    if (prop.major != 10) return TRACER_ERR_NO_SUITABLE_GPU;
    if (cudaSetDevice(cuda_device) != cudaSuccess) return TRACER_ERR_NO_SUITABLE_GPU;
    tracer_ctx* c = new tracer_ctx();
    c->device = cuda_device;
    c->sm_count = prop.multiProcessorCount;
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = dalloc(c->stats, C_COUNT);
    if (e == cudaSuccess) e = dalloc(c->status, 1);
    if (e == cudaSuccess) e = dalloc(c->wf_count, 4);
    if (e == cudaSuccess) e = cudaMallocHost(&c->pinned_counts, sizeof(uint32_t) * kCountSlots);
    if (e == cudaSuccess) {
        c->count_events.resize(kCountSlots, nullptr);
        for (auto& ev : c->count_events)
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaEventCreate(&c->prof_begin);
    if (e == cudaSuccess) e = cudaEventCreate(&c->prof_end);
    if (e != cudaSuccess) {
        tracer_destroy(c);
        return e == cudaErrorMemoryAllocation ? TRACER_ERR_OOM : TRACER_ERR_CUDA;
    }
    *out = c;
    return TRACER_OK;
}

void tracer_destroy(tracer_ctx* c)
{
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->pending && c->done) wait_event(c, c->done);
    c->scene.release();
    c->batch.release();
    c->adj.release();
    c->slot[0].release();
    c->slot[1].release();
    c->acc_sum.release();
    c->acc_disp[0].release();
    c->acc_disp[1].release();
    c->pres_src[0].release();
    c->pres_src[1].release();
    c->pres_out.release();
    c->batch_slots.release();
    c->b_rgba8.release();
    c->b_rgba32f.release();
    c->b_hit.release();
    if (c->pinned_slots) cudaFreeHost(c->pinned_slots);
    if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
    if (c->graph) cudaGraphDestroy(c->graph);
    c->rgba8.release();
    c->rgba32f.release();
    c->hit.release();
    c->linear.release();
    c->stats.release();
    c->status.release();
    release_wavefront(c);
    c->wf_count.release();
    if (c->pinned_counts) cudaFreeHost(c->pinned_counts);
    for (auto ev : c->count_events)
        if (ev) cudaEventDestroy(ev);
    for (auto ev : c->prof_events)
        if (ev) cudaEventDestroy(ev);
    if (c->prof_begin) cudaEventDestroy(c->prof_begin);
    if (c->prof_end) cudaEventDestroy(c->prof_end);
    if (c->done) cudaEventDestroy(c->done);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

const char* tracer_last_error(const tracer_ctx* c) { return c ? c->err.c_str() : "null context"; }

int tracer_set_traversal_limit(tracer_ctx* c, uint32_t steps)
{
    if (!c) return TRACER_ERR_INVALID_ARG;
    int r = finish(c);
    if (r != TRACER_OK) return r;
    c->trav_cap = steps;
    return TRACER_OK;
}

int tracer_set_adjoint_hit_log(tracer_ctx* c, uint64_t max_bytes)
{
    if (!c) return TRACER_ERR_INVALID_ARG;
    c->adj_log_limit = max_bytes;
    if (max_bytes == 0) c->adj.log.release();
    return TRACER_OK;
}

int tracer_set_edge_sampling(tracer_ctx* c, uint32_t samples_per_edge)
{
    if (!c) return TRACER_ERR_INVALID_ARG;
    if (samples_per_edge > 1024) return fail(c, TRACER_ERR_INVALID_ARG, "at most 1024 samples per edge");
    c->edge_samples = samples_per_edge;
    return TRACER_OK;
}

int tracer_set_timeout(tracer_ctx* c, uint32_t ms)
{
    if (!c || ms == 0) return TRACER_ERR_INVALID_ARG;
    c->timeout_ms = ms;
    return TRACER_OK;
}

int tracer_upload_scene(tracer_ctx* c, const tracer_scene_desc* d)
{
    if (!c) return TRACER_ERR_INVALID_ARG;
    if (!d) return fail(c, TRACER_ERR_INVALID_ARG, "null scene description");
    if (d->num_triangles && !d->triangles) return fail(c, TRACER_ERR_INVALID_ARG, "null triangle array");
    if (d->num_spheres && !d->spheres) return fail(c, TRACER_ERR_INVALID_ARG, "null sphere array");
    if (d->num_planes && !d->planes) return fail(c, TRACER_ERR_INVALID_ARG, "null plane array");
    if (d->num_materials && !d->materials) return fail(c, TRACER_ERR_INVALID_ARG, "null material array");
    if (d->bvh != TRACER_BVH_NONE && d->bvh != TRACER_BVH_MEDIAN && d->bvh != TRACER_BVH_SAH)
        return fail(c, TRACER_ERR_INVALID_ARG, "unknown BVH kind %d", d->bvh);
    if ((uint64_t)d->num_triangles + d->num_spheres + d->num_planes >= 0xFFFFFFFFull)
        return fail(c, TRACER_ERR_INVALID_ARG, "too many primitives");
    for (uint32_t i = 0; i < d->num_triangles; ++i)
        if (d->triangles[i].material >= d->num_materials)
            return fail(c, TRACER_ERR_INVALID_ARG, "triangle %u uses material %u of %u", i, d->triangles[i].material,
                        d->num_materials);
    int r = finish(c);
    if (r != TRACER_OK) return r;
    cudaSetDevice(c->device);
    SceneBuffers& s = c->scene;
    s.release();
    s.nt = d->num_triangles;
    s.nm = d->num_materials;
    s.ns = d->num_spheres;
    s.np = d->num_planes;
    s.bvh = d->bvh != TRACER_BVH_NONE;

    // Triangles in traversal order: (v0, material) (v1 - v0, id) (v2 - v0, 0)
    std::vector<tracer_bvh_node> tnodes, snodes;
    std::vector<uint32_t> tidx, sidx;
    uint32_t tdepth = 0, sdepth = 0;
    if (s.bvh && s.nt) {
        r = prepare_bvh(c, d->bvh, TRACER_PRIM_TRIANGLE, d->triangles, s.nt, d->leaf_size, d->sah_bins, d->tri_nodes,
                        d->num_tri_nodes, d->tri_prim_index, tnodes, tidx, tdepth);
        if (r != TRACER_OK) return r;
    }
    if (s.bvh && s.ns) {
        r = prepare_bvh(c, d->bvh, TRACER_PRIM_SPHERE, d->spheres, s.ns, d->leaf_size, d->sah_bins, d->sphere_nodes,
                        d->num_sphere_nodes, d->sphere_prim_index, snodes, sidx, sdepth);
        if (r != TRACER_OK) return r;
    }
    std::vector<float4> tri(3 * (size_t)s.nt);
    for (uint32_t k = 0; k < s.nt; ++k) {
        const uint32_t i = s.bvh ? tidx[k] : k;
        const tracer_triangle& t = d->triangles[i];
        float m, id;
        std::memcpy(&m, &t.material, 4);
        std::memcpy(&id, &i, 4);
        tri[3 * k + 0] = make_float4(t.v0[0], t.v0[1], t.v0[2], m);
        tri[3 * k + 1] = make_float4(t.v1[0] - t.v0[0], t.v1[1] - t.v0[1], t.v1[2] - t.v0[2], id);
        tri[3 * k + 2] = make_float4(t.v2[0] - t.v0[0], t.v2[1] - t.v0[1], t.v2[2] - t.v0[2], 0.0f);
    }
    std::vector<float4> geo(s.ns);
    std::vector<uint32_t> sid(s.ns), emit;
    for (uint32_t k = 0; k < s.ns; ++k) {
        const uint32_t i = s.bvh ? sidx[k] : k;
        const tracer_sphere& q = d->spheres[i];
        geo[k] = make_float4(q.P[0], q.P[1], q.P[2], q.r);
        sid[k] = i;
    }
    for (uint32_t i = 0; i < s.ns; ++i) {
        const float* em = d->spheres[i].mat.emissive;
        if (!(em[0] == 0.0f && em[1] == 0.0f && em[2] == 0.0f)) emit.push_back(i);
    }
    s.ne = (uint32_t)emit.size();
    s.n_tri_nodes = (uint32_t)tnodes.size();
    s.n_sph_nodes = (uint32_t)snodes.size();
    s.depth = tdepth > sdepth ? tdepth : sdepth;
    // the same BVHs as 4-wide nodes for the wavefront traversal
    std::vector<WideNode> twide, swide;
    uint32_t twd = 0, swd = 0;
    const bool wide_ok = collapse_wide4(tnodes.data(), (uint32_t)tnodes.size(), twide, &twd) &&
                         collapse_wide4(snodes.data(), (uint32_t)snodes.size(), swide, &swd);
    s.wide_depth = twd > swd ? twd : swd;
    std::vector<tracer_bvh_node> tenc, senc;
    if (!encode_refs(tnodes.data(), (uint32_t)tnodes.size(), tenc) ||
        !encode_refs(snodes.data(), (uint32_t)snodes.size(), senc))
        return fail(c, TRACER_ERR_BAD_BVH, "a BVH leaf holds more than 64 primitives or starts beyond 2^25");
    std::vector<Cw8Node> cw8;
    std::vector<float4> cw8_prims;
    uint32_t cw8_depth = 0;
    const bool cw8_ok = s.bvh && s.nt > 0 && s.ns == 0 && make_cw8(tnodes, tri, cw8, cw8_prims, cw8_depth);

    cudaError_t e = upload(s.tri, tri.data(), tri.size());
    if (e == cudaSuccess) e = upload(s.mats, reinterpret_cast<const float4*>(d->materials), 3 * (size_t)s.nm);
    if (e == cudaSuccess) e = upload(s.sph_geo, geo.data(), geo.size());
    if (e == cudaSuccess) e = upload(s.sph_id, sid.data(), sid.size());
    if (e == cudaSuccess) e = upload(s.sph_rec, reinterpret_cast<const float4*>(d->spheres), 4 * (size_t)s.ns);
    if (e == cudaSuccess) e = upload(s.planes, reinterpret_cast<const float4*>(d->planes), 4 * (size_t)s.np);
    if (e == cudaSuccess) e = upload(s.emit, emit.data(), emit.size());
    if (e == cudaSuccess)
        e = upload(s.tri_nodes, reinterpret_cast<const float4*>(tnodes.data()), 2 * tnodes.size());
    if (e == cudaSuccess)
        e = upload(s.sph_nodes, reinterpret_cast<const float4*>(snodes.data()), 2 * snodes.size());
    if (e == cudaSuccess) e = upload(s.tri_enc, reinterpret_cast<const float4*>(tenc.data()), 2 * tenc.size());
    if (e == cudaSuccess) e = upload(s.sph_enc, reinterpret_cast<const float4*>(senc.data()), 2 * senc.size());
    if (e == cudaSuccess && wide_ok)
        e = upload(s.tri_wide, reinterpret_cast<const float4*>(twide.data()), 8 * twide.size());
    if (e == cudaSuccess && wide_ok)
        e = upload(s.sph_wide, reinterpret_cast<const float4*>(swide.data()), 8 * swide.size());
    if (e == cudaSuccess && cw8_ok) e = upload(s.tri_cw8, reinterpret_cast<const float4*>(cw8.data()), 6 * cw8.size());
    if (e == cudaSuccess && cw8_ok) e = upload(s.tri_cw8_prims, cw8_prims.data(), cw8_prims.size());
    if (e != cudaSuccess) {
        s.release();
        return cuda_fail(c, e, "scene upload");
    }
    s.wide = wide_ok;
    s.cw8 = cw8_ok;
    s.cw8_depth = cw8_depth;
    s.loaded = true;
    ++c->scene_version;
    return TRACER_OK;
}

int tracer_set_materials(tracer_ctx* c, const tracer_material* mats, uint32_t n)
{
    if (!c) return TRACER_ERR_INVALID_ARG;
    if (!c->scene.loaded) return fail(c, TRACER_ERR_NO_SCENE, "no scene uploaded");
    if (!mats || n != c->scene.nm) return fail(c, TRACER_ERR_INVALID_ARG, "material count %u != %u", n, c->scene.nm);
    int r = finish(c);
    if (r != TRACER_OK) return r;
    cudaError_t e = cudaMemcpy(c->scene.mats.p, mats, sizeof(tracer_material) * n, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(c, e, "material update");
    ++c->scene_version;
    return TRACER_OK;
}

int tracer_trace(tracer_ctx* c, const tracer_frame* f, const tracer_trace_params* p, void* cuda_stream)
{
    if (!c) return TRACER_ERR_INVALID_ARG;
    if (!f || !p) return fail(c, TRACER_ERR_INVALID_ARG, "null frame or params");
    if (!c->scene.loaded) return fail(c, TRACER_ERR_NO_SCENE, "no scene uploaded");
    if (p->width == 0 || p->height == 0 || p->width > 32768 || p->height > 32768)
        return fail(c, TRACER_ERR_NO_SUITABLE_SURFACE, "image size %ux%u not supported", p->width, p->height);
    if (p->spp == 0 || p->max_depth == 0 || p->max_depth > 1024 || p->spp > 1u << 20)
        return fail(c, TRACER_ERR_INVALID_ARG, "spp %u / max_depth %u out of range", p->spp, p->max_depth);
    if (p->tie_mode != TRACER_TIES_REFERENCE && p->tie_mode != TRACER_TIES_STRICT)
        return fail(c, TRACER_ERR_INVALID_ARG, "unknown tie mode %d", p->tie_mode);
    if (p->tie_mode == TRACER_TIES_REFERENCE && c->scene.bvh)
        return fail(c, TRACER_ERR_INVALID_ARG, "reference ties depend on scan order and need a linear-scan scene");
    // AUTO: the wavefront on BVH scenes with enough path bounces in flight --
    // from 2^16 where the scene has an 8-wide BVH (its traversal, in the
    // extend and finishing kernels, wins even on small frames), from 2^22
    // otherwise; the plain kernel on linear-scan scenes and small frames.
    // Measured (plain / wavefront ms), 8-wide: c3 scene 128^2 x 4 spp x
    // depth 4 (2^18 bounces) 0.48 / 0.30, 256^2 x 4 x 4 0.59 / 0.38, 512^2
    // 1.42 / 0.91; c1 scene 128^2 x 4 x 8 2.63 / 1.63, 256^2 x 4 x 8 2.95 /
    // 1.83, 640x360 x 4 x 8 8.06 / 3.08, 1920x1080 x 16 x 8 222 / 58; c4
    // scene 256^2 x 4 x 12 6.22 / 3.80.  Binary only: c0 (spheres) 512^2 x 1
    // x 2 0.067 / 0.118; the reference's own 10-primitive frame (linear) 1.6
    // / 2.2.
    const uint64_t bounces = (uint64_t)p->width * p->height * p->spp * p->max_depth;
    const bool cw8_auto = c->scene.cw8 && (p->bvh_width == 0 || p->bvh_width == 8);
    const int kernel = p->kernel != TRACER_KERNEL_AUTO ? p->kernel
                       : (c->scene.bvh && bounces >= (cw8_auto ? (1ull << 16) : (1ull << 22)))
                           ? TRACER_KERNEL_WAVEFRONT
                           : TRACER_KERNEL_PLAIN;
    if (kernel != TRACER_KERNEL_PLAIN && kernel != TRACER_KERNEL_WAVEFRONT)
        return fail(c, TRACER_ERR_INVALID_ARG, "unknown kernel %d", p->kernel);
    uint32_t block = p->block ? p->block : 128;
    if (block % 32 != 0 || block < 32 || block > 256)
        return fail(c, TRACER_ERR_INVALID_ARG, "block %u must be a multiple of 32 in [32, 256]", block);
    if (kernel == TRACER_KERNEL_WAVEFRONT && block != 64 && block != 128 && block != 256)
        return fail(c, TRACER_ERR_INVALID_ARG, "wavefront block must be 64, 128 or 256");
    uint32_t need = c->scene.bvh ? (c->scene.depth > 1 ? c->scene.depth : 1) : 0;
    uint32_t stack = p->stack_depth ? p->stack_depth : need;
    if (c->scene.bvh && stack < need)
        return fail(c, TRACER_ERR_STACK_OVERFLOW, "stack depth %u below the BVH depth %u", stack, need);
    if ((size_t)stack * 256 * 8 > 200 * 1024)
        return fail(c, TRACER_ERR_INVALID_ARG, "stack depth %u exceeds shared memory", stack);
    const uint32_t mask = p->aov_mask ? p->aov_mask : (1u << TRACER_AOV_RGBA8);
    if (mask & ~((1u << TRACER_AOV_RGBA8) | (1u << TRACER_AOV_RGBA32F) | (1u << TRACER_AOV_PRIMARY_HIT) |
                 (1u << TRACER_AOV_STATS) | (1u << TRACER_AOV_LINEAR)))
        return fail(c, TRACER_ERR_NO_SUITABLE_SURFACE, "unknown AOV in mask 0x%x", mask);

    int r = finish(c);
    if (r != TRACER_OK) return r;
    cudaSetDevice(c->device);
    const size_t npx = (size_t)p->width * p->height;
    cudaError_t e = cudaSuccess;
    if (mask & (1u << TRACER_AOV_RGBA8)) e = dalloc(c->rgba8, npx);
    if (e == cudaSuccess && (mask & (1u << TRACER_AOV_RGBA32F))) e = dalloc(c->rgba32f, npx);
    if (e == cudaSuccess && (mask & (1u << TRACER_AOV_PRIMARY_HIT))) e = dalloc(c->hit, npx);
    if (e == cudaSuccess && (mask & (1u << TRACER_AOV_LINEAR))) e = dalloc(c->linear, npx);
    if (e != cudaSuccess) return cuda_fail(c, e, "image allocation");
    c->width = p->width;
    c->height = p->height;
    c->last_mask = mask;

    TraceArgs a;
    std::memset(&a, 0, sizeof a);
    const SceneBuffers& s = c->scene;
    a.sc = DevScene{s.tri.p, s.mats.p, s.sph_geo.p, s.sph_id.p, s.sph_rec.p, s.planes.p, s.emit.p, s.tri_nodes.p,
                    s.sph_nodes.p, s.nt, s.nm, s.ns, s.np, s.ne, s.n_tri_nodes, s.n_sph_nodes,
                    s.tri_wide.p, s.sph_wide.p, s.tri_enc.p, s.sph_enc.p, s.tri_cw8.p, s.tri_cw8_prims.p};
    a.fr.aspect = f->aspect_ratio;
    a.fr.seed = f->seed;
    const tracer_camera& cam = f->camera;
    a.fr.cpos = V3{cam.pos[0], cam.pos[1], cam.pos[2]};
    a.fr.cdir = V3{cam.dir[0], cam.dir[1], cam.dir[2]};
    a.fr.cright = V3{cam.right[0], cam.right[1], cam.right[2]};
    a.fr.cup = V3{cam.up[0], cam.up[1], cam.up[2]};
    a.width = p->width;
    a.height = p->height;
    a.spp = p->spp;
    a.max_depth = p->max_depth;
    a.rr_start = p->rr_start;
    a.sky = V3{p->sky[0], p->sky[1], p->sky[2]};
    a.sky_on = !(p->sky[0] == 0.0f && p->sky[1] == 0.0f && p->sky[2] == 0.0f);
    a.stack_depth = stack;
    const uint32_t nn = s.n_tri_nodes > s.n_sph_nodes ? s.n_tri_nodes : s.n_sph_nodes;
    a.trav_limit = trav_limit(c, nn);
    a.rgba8 = (mask & (1u << TRACER_AOV_RGBA8)) ? c->rgba8.p : nullptr;
    a.rgba32f = (mask & (1u << TRACER_AOV_RGBA32F)) ? c->rgba32f.p : nullptr;
    a.hit = (mask & (1u << TRACER_AOV_PRIMARY_HIT)) ? c->hit.p : nullptr;
    a.linear = (mask & (1u << TRACER_AOV_LINEAR)) ? c->linear.p : nullptr;
    a.stats = c->stats.p;
    a.status = c->status.p;
    const int stats = (p->stats || (mask & (1u << TRACER_AOV_STATS))) ? 1 : 0;
    if (stats) c->last_mask |= 1u << TRACER_AOV_STATS;
    cudaStream_t st = cuda_stream ? static_cast<cudaStream_t>(cuda_stream) : c->stream;
    e = cudaMemsetAsync(c->stats.p, 0, sizeof(unsigned long long) * C_COUNT, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->status.p, 0, sizeof(int), st);
    if (e != cudaSuccess) return cuda_fail(c, e, "trace set-up");
    c->last_kernel = kernel;
    c->last_rounds = 0;
    c->last_prof_rounds = 0;
    c->last_round_entries = 0;
    c->last_finish = false;
    c->last_launches = 0;
    if (c->profiling) cudaEventRecord(c->prof_begin, st);

    if (kernel == TRACER_KERNEL_PLAIN) {
        LaunchConfig lc{block, stats, p->tie_mode, s.bvh ? 1 : 0};
        e = launch_plain(a, lc, st);
        c->last_launches = 1;
    } else {
        e = ensure_wavefront(c, npx);
        if (e != cudaSuccess) return cuda_fail(c, e, "wavefront state allocation");
        a.pixel_base = 0;
        a.num_slots = (uint32_t)npx;
        WfConfig wc;
        std::memset(&wc, 0, sizeof wc);
        wc.tie = p->tie_mode;
        wc.bvh = s.bvh ? 1 : 0;
        wc.stats = stats;
        wc.has_emitters = s.ne > 0;
        wc.block = p->block ? p->block : 128;
        uint32_t wstack = stack;
        r = pick_width(c, p, wstack, wc.wide);
        if (r != TRACER_OK) return r;
        a.stack_depth = wstack;
        if (wc.wide == WF_WIDTH_8) wc.cw8_stack = s.cw8_depth;
        if (wc.wide != WF_WIDTH_8) a.sc.tri_cw8 = a.sc.tri_cw8_prims = nullptr;  // finishing kernel: binary too
        r = run_wavefront(c, a, wc, npx, (uint64_t)p->spp * p->max_depth + 1, wstack, p->wavefront, p->tail_paths, st);
        if (r != TRACER_OK) return r;
    }
    if (c->profiling) cudaEventRecord(c->prof_end, st);
    if (e == cudaSuccess) e = cudaEventRecord(c->done, st);
    if (e != cudaSuccess) return cuda_fail(c, e, "trace launch");
    c->pending = true;
    return TRACER_OK;
}

int tracer_measure_l2_read(tracer_ctx* c, size_t bytes, uint32_t passes, double* gbs)
{
    if (!c || !gbs || passes == 0 || bytes < 16 || bytes % 16) return TRACER_ERR_INVALID_ARG;
    *gbs = 0.0;
    cudaSetDevice(c->device);
    int r = finish(c);
    if (r != TRACER_OK) return r;
    const uint32_t blocks = (uint32_t)c->sm_count * 8;
    DevBuf<unsigned char> buf;
    DevBuf<uint32_t> sink;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    cudaError_t e = dalloc(buf, bytes);
    if (e == cudaSuccess) e = dalloc(sink, (size_t)blocks * 256);
    if (e == cudaSuccess) e = cudaMemsetAsync(buf.p, 1, bytes, c->stream);
    if (e == cudaSuccess) e = cudaEventCreate(&ev[0]);
    if (e == cudaSuccess) e = cudaEventCreate(&ev[1]);
    // one untimed launch brings the buffer into L2
    if (e == cudaSuccess) e = launch_l2_read(buf.p, bytes, 1, sink.p, blocks, c->stream);
    if (e == cudaSuccess) e = cudaEventRecord(ev[0], c->stream);
    if (e == cudaSuccess) e = launch_l2_read(buf.p, bytes, passes, sink.p, blocks, c->stream);
    if (e == cudaSuccess) e = cudaEventRecord(ev[1], c->stream);
    if (e == cudaSuccess) {
        r = wait_event(c, ev[1]);
        float ms = 0.0f;
        if (r == TRACER_OK) e = cudaEventElapsedTime(&ms, ev[0], ev[1]);
        if (r == TRACER_OK && e == cudaSuccess && ms > 0.0f) *gbs = (double)bytes * passes / (ms * 1e-3) / 1e9;
    }
    for (cudaEvent_t x : ev)
        if (x) cudaEventDestroy(x);
    buf.release();
    sink.release();
    if (e != cudaSuccess) return cuda_fail(c, e, "L2 read measurement");
    return r;
}

int tracer_set_profiling(tracer_ctx* c, int enable)
{
    if (!c) return TRACER_ERR_INVALID_ARG;
    c->profiling = enable != 0;
    return TRACER_OK;
}

int tracer_last_timings(tracer_ctx* c, tracer_timings* out)
{
    if (!c || !out) return TRACER_ERR_INVALID_ARG;
    int r = finish(c);
    if (r != TRACER_OK) return r;
    std::memset(out, 0, sizeof *out);
    out->rounds = c->last_rounds;
    out->launches = c->last_launches;
    if (!c->profiling) return fail(c, TRACER_ERR_INVALID_ARG, "profiling is off (tracer_set_profiling)");
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, c->prof_begin, c->prof_end) == cudaSuccess) out->total_ms = ms;
    if (c->last_kernel == TRACER_KERNEL_WAVEFRONT) {
        for (uint32_t i = 0; i < c->last_prof_rounds && 3 * (size_t)i + 2 < c->prof_events.size(); ++i) {
            if (cudaEventElapsedTime(&ms, c->prof_events[3 * i], c->prof_events[3 * i + 1]) == cudaSuccess)
                out->extend_ms += ms;
            if (cudaEventElapsedTime(&ms, c->prof_events[3 * i + 1], c->prof_events[3 * i + 2]) == cudaSuccess)
                out->shade_ms += ms;
        }
        const size_t f = c->last_prof_rounds;
        if (c->last_finish && 3 * f + 1 < c->prof_events.size() &&
            cudaEventElapsedTime(&ms, c->prof_events[3 * f], c->prof_events[3 * f + 1]) == cudaSuccess)
            out->finish_ms = ms;
    }
    return TRACER_OK;
}

int tracer_last_rounds(tracer_ctx* c, tracer_round_info* out, uint32_t cap, uint32_t* n)
{
    if (!c || !n || (cap && !out)) return TRACER_ERR_INVALID_ARG;
    *n = 0;
    int r = finish(c);
    if (r != TRACER_OK) return r;
    if (!c->profiling) return fail(c, TRACER_ERR_INVALID_ARG, "profiling is off (tracer_set_profiling)");
    if (c->last_kernel != TRACER_KERNEL_WAVEFRONT || c->last_round_entries == 0) return TRACER_OK;
    const uint32_t rounds = c->last_prof_rounds;
    const uint32_t entries = c->last_round_entries < rounds + (c->last_finish ? 1u : 0u)
                                 ? c->last_round_entries
                                 : rounds + (c->last_finish ? 1u : 0u);
    std::vector<uint32_t> paths(entries);
    cudaError_t e = cudaMemcpy(paths.data(), c->round_paths.p, sizeof(uint32_t) * entries, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(c, e, "reading round statistics");
    *n = entries;
    for (uint32_t i = 0; i < entries && i < cap; ++i) {
        tracer_round_info& o = out[i];
        o.paths = paths[i];
        o.finish = (c->last_finish && i == rounds) ? 1u : 0u;
        o.extend_ms = 0.0f;
        o.shade_ms = 0.0f;
        float ms = 0.0f;
        if (3 * (size_t)i + 1 < c->prof_events.size() &&
            cudaEventElapsedTime(&ms, c->prof_events[3 * i], c->prof_events[3 * i + 1]) == cudaSuccess)
            o.extend_ms = ms;
        if (!o.finish && 3 * (size_t)i + 2 < c->prof_events.size() &&
            cudaEventElapsedTime(&ms, c->prof_events[3 * i + 1], c->prof_events[3 * i + 2]) == cudaSuccess)
            o.shade_ms = ms;
    }
    return TRACER_OK;
}

int tracer_synchronize(tracer_ctx* c)
{
    if (!c) return TRACER_ERR_INVALID_ARG;
    cudaSetDevice(c->device);
    return finish(c);
}

static int aov_info(tracer_ctx* c, int aov, void** ptr, size_t* bytes)
{
    const size_t npx = (size_t)c->width * c->height;
    const uint32_t bit = aov >= 0 && aov < 32 ? (1u << aov) : 0;
    if (!bit || !(c->last_mask & bit) || c->width == 0)
        return fail(c, TRACER_ERR_NO_SUITABLE_SURFACE, "AOV %d was not produced by the last trace", aov);
    switch (aov) {
    case TRACER_AOV_RGBA8: *ptr = c->rgba8.p; *bytes = npx * 4; break;
    case TRACER_AOV_RGBA32F: *ptr = c->rgba32f.p; *bytes = npx * 16; break;
    case TRACER_AOV_PRIMARY_HIT: *ptr = c->hit.p; *bytes = npx * 8; break;
    case TRACER_AOV_LINEAR: *ptr = c->linear.p; *bytes = npx * 16; break;
    case TRACER_AOV_STATS: *ptr = c->stats.p; *bytes = sizeof(tracer_stats); break;
    default: return fail(c, TRACER_ERR_NO_SUITABLE_SURFACE, "unknown AOV %d", aov);
    }
    return TRACER_OK;
}

int tracer_readback(tracer_ctx* c, int aov, void* dst, size_t bytes)
{
    if (!c) return TRACER_ERR_INVALID_ARG;
    if (!dst) return fail(c, TRACER_ERR_INVALID_ARG, "null destination");
    cudaSetDevice(c->device);
    int r = finish(c);
    if (r != TRACER_OK) return r;
    void* src;
    size_t n;
    r = aov_info(c, aov, &src, &n);
    if (r != TRACER_OK) return r;
    if (bytes != n) return fail(c, TRACER_ERR_INVALID_ARG, "AOV %d holds %zu bytes, %zu requested", aov, n, bytes);
    cudaError_t e = cudaMemcpy(dst, src, n, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(c, e, "readback");
    return TRACER_OK;
}

int tracer_device_image(tracer_ctx* c, int aov, void** ptr, size_t* bytes)
{
    if (!c) return TRACER_ERR_INVALID_ARG;
    if (!ptr || !bytes) return fail(c, TRACER_ERR_INVALID_ARG, "null output");
    return aov_info(c, aov, ptr, bytes);
}

}  // extern "C"

// ------------------------------------------------------- no-alloc entry point
// Scratch of tracer_trace_noalloc: the wavefront path state, both queues, the
// queue counters and the status/statistics words for up to
// TRACER_NOALLOC_MAX_PIXELS pixels, in one fixed array so that the call never
// allocates.  Region sizes are multiples of 256 bytes, so each region stays
// 256-byte aligned.
namespace {
constexpr size_t kNaPix = TRACER_NOALLOC_MAX_PIXELS;
constexpr size_t kNaF4 = kNaPix * sizeof(float4);   // one float4 / uint4 per pixel
constexpr size_t kNaU32 = kNaPix * sizeof(uint32_t);
constexpr size_t kNaOffRayO = 0;
constexpr size_t kNaOffRayD = kNaOffRayO + kNaF4;
constexpr size_t kNaOffHit = kNaOffRayD + kNaF4;
constexpr size_t kNaOffAcc = kNaOffHit + kNaF4;
constexpr size_t kNaOffMask = kNaOffAcc + kNaF4;
constexpr size_t kNaOffAccum = kNaOffMask + kNaF4;
constexpr size_t kNaOffPrim0 = kNaOffAccum + kNaF4;
constexpr size_t kNaOffQ0 = kNaOffPrim0 + kNaU32;
constexpr size_t kNaOffQ1 = kNaOffQ0 + kNaU32;
constexpr size_t kNaOffCount = kNaOffQ1 + kNaU32;     // 4 x u32
constexpr size_t kNaOffStats = kNaOffCount + 256;     // C_COUNT x u64
constexpr size_t kNaOffStatus = kNaOffStats + 256;    // int
constexpr size_t kNaBytes = kNaOffStatus + 256;
static_assert(kNaF4 % 256 == 0 && kNaU32 % 256 == 0, "regions must keep 256-byte alignment");
static_assert(C_COUNT * sizeof(unsigned long long) <= 256, "statistics region too small");
constexpr int kNaMaxDevices = 64;

std::mutex g_noalloc_mutex;
void* g_noalloc_addr[kNaMaxDevices] = {};
}  // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaBytes];

// Device address of the scratch array on the current device, looked up once
// per device (the host-side symbol is only a stand-in for it).
static int noalloc_scratch(tracer_ctx* c, unsigned char** out)
{
    if (c->device < 0 || c->device >= kNaMaxDevices)
        return fail(c, TRACER_ERR_NO_SUITABLE_GPU, "device %d beyond the no-alloc set-up table", c->device);
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_addr[c->device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) return cuda_fail(c, e, "looking up the no-alloc scratch address");
        g_noalloc_addr[c->device] = p;
    }
    *out = static_cast<unsigned char*>(g_noalloc_addr[c->device]);
    return TRACER_OK;
}

extern "C" int tracer_trace_noalloc(tracer_ctx* c, const tracer_frame* f, const tracer_trace_params* p,
                                    void* rgba8_out, void* rgba32f_out, void* cuda_stream)
{
    if (!c) return TRACER_ERR_INVALID_ARG;
    if (!f || !p) return fail(c, TRACER_ERR_INVALID_ARG, "null frame or params");
    if (!rgba8_out && !rgba32f_out) return fail(c, TRACER_ERR_INVALID_ARG, "no output buffer given");
    if (!c->scene.loaded) return fail(c, TRACER_ERR_NO_SCENE, "no scene uploaded");
    if (p->width == 0 || p->height == 0 || (uint64_t)p->width * p->height > kNaPix)
        return fail(c, TRACER_ERR_NO_SUITABLE_SURFACE,
                    "image %ux%u exceeds the no-alloc limit of %u pixels (use tracer_trace)", p->width, p->height,
                    TRACER_NOALLOC_MAX_PIXELS);
    if (p->spp == 0 || p->max_depth == 0 || (uint64_t)p->spp * p->max_depth > TRACER_NOALLOC_MAX_ROUNDS)
        return fail(c, TRACER_ERR_INVALID_ARG, "spp %u x max_depth %u exceeds the no-alloc limit of %u rounds",
                    p->spp, p->max_depth, TRACER_NOALLOC_MAX_ROUNDS);
    if (p->tie_mode != TRACER_TIES_REFERENCE && p->tie_mode != TRACER_TIES_STRICT)
        return fail(c, TRACER_ERR_INVALID_ARG, "unknown tie mode %d", p->tie_mode);
    if (p->tie_mode == TRACER_TIES_REFERENCE && c->scene.bvh)
        return fail(c, TRACER_ERR_INVALID_ARG, "reference ties depend on scan order and need a linear-scan scene");
    if (p->bvh_width != 0 && p->bvh_width != 2)
        return fail(c, TRACER_ERR_INVALID_ARG, "bvh_width %u: the no-alloc trace runs the binary traversal only (0 or 2)",
                    p->bvh_width);
    const SceneBuffers& s = c->scene;
    const uint32_t need = s.bvh ? (s.depth > 1 ? s.depth : 1) : 0;
    const uint32_t stack = p->stack_depth ? p->stack_depth : need;
    if (s.bvh && stack < need)
        return fail(c, TRACER_ERR_STACK_OVERFLOW, "stack depth %u below the BVH depth %u", stack, need);
    if ((size_t)stack * 256 * 8 > 200 * 1024)
        return fail(c, TRACER_ERR_INVALID_ARG, "stack depth %u exceeds shared memory", stack);
    if (cudaSetDevice(c->device) != cudaSuccess) return fail(c, TRACER_ERR_CUDA, "cannot select device %d", c->device);
    unsigned char* base = nullptr;
    int r = noalloc_scratch(c, &base);
    if (r != TRACER_OK) return r;

    TraceArgs a;
    std::memset(&a, 0, sizeof a);
    a.sc = DevScene{s.tri.p, s.mats.p, s.sph_geo.p, s.sph_id.p, s.sph_rec.p, s.planes.p, s.emit.p, s.tri_nodes.p,
                    s.sph_nodes.p, s.nt, s.nm, s.ns, s.np, s.ne, s.n_tri_nodes, s.n_sph_nodes,
                    s.tri_wide.p, s.sph_wide.p, s.tri_enc.p, s.sph_enc.p, nullptr, nullptr};  // binary traversal only
    a.fr.aspect = f->aspect_ratio;
    a.fr.seed = f->seed;
    a.fr.cpos = V3{f->camera.pos[0], f->camera.pos[1], f->camera.pos[2]};
    a.fr.cdir = V3{f->camera.dir[0], f->camera.dir[1], f->camera.dir[2]};
    a.fr.cright = V3{f->camera.right[0], f->camera.right[1], f->camera.right[2]};
    a.fr.cup = V3{f->camera.up[0], f->camera.up[1], f->camera.up[2]};
    a.width = p->width;
    a.height = p->height;
    a.spp = p->spp;
    a.max_depth = p->max_depth;
    a.rr_start = p->rr_start;
    a.sky = V3{p->sky[0], p->sky[1], p->sky[2]};
    a.sky_on = !(p->sky[0] == 0.0f && p->sky[1] == 0.0f && p->sky[2] == 0.0f);
    a.stack_depth = stack;
    const uint32_t nn = s.n_tri_nodes > s.n_sph_nodes ? s.n_tri_nodes : s.n_sph_nodes;
    a.trav_limit = trav_limit(c, nn);
    a.rgba8 = static_cast<uchar4*>(rgba8_out);
    a.rgba32f = static_cast<float4*>(rgba32f_out);
    a.hit = nullptr;
    a.stats = reinterpret_cast<unsigned long long*>(base + kNaOffStats);
    a.status = reinterpret_cast<int*>(base + kNaOffStatus);
    a.pixel_base = 0;
    a.num_slots = p->width * p->height;

    WfState ws{reinterpret_cast<float4*>(base + kNaOffRayO), reinterpret_cast<float4*>(base + kNaOffRayD),
               reinterpret_cast<uint4*>(base + kNaOffHit), reinterpret_cast<float4*>(base + kNaOffAcc),
               reinterpret_cast<float4*>(base + kNaOffMask), reinterpret_cast<float4*>(base + kNaOffAccum),
               reinterpret_cast<uint32_t*>(base + kNaOffPrim0),
               {reinterpret_cast<uint32_t*>(base + kNaOffQ0), reinterpret_cast<uint32_t*>(base + kNaOffQ1)},
               reinterpret_cast<uint32_t*>(base + kNaOffCount), nullptr};
    WfConfig wc;
    std::memset(&wc, 0, sizeof wc);
    wc.tie = p->tie_mode;
    wc.bvh = s.bvh ? 1 : 0;
    wc.stats = 0;
    wc.has_emitters = s.ne > 0;
    wc.block = 128;
    int per = wf_extend_blocks_per_sm(wc, stack);
    if (per <= 0) return fail(c, TRACER_ERR_INVALID_ARG, "extend kernel cannot be resident (stack %u)", stack);
    if (p->wavefront && (int)p->wavefront < per) per = (int)p->wavefront;
    wc.extend_grid = (uint32_t)(per * c->sm_count);
    const size_t npx = (size_t)p->width * p->height;
    wc.shade_grid = (uint32_t)((npx + 255) / 256);

    cudaStream_t st = cuda_stream ? static_cast<cudaStream_t>(cuda_stream) : c->stream;
    // The status word starts at zero; the generate kernel resets the queue
    // counters; statistics are not collected here.
    cudaError_t e = cudaMemsetAsync(a.status, 0, sizeof(int), st);
    if (e == cudaSuccess) e = wf_launch_generate(a, ws, wc, st);
    // No queue length is read back to the host.  With fewer pixels than the
    // point below which tracer_trace runs no round (tail_paths, or with the
    // automatic threshold the extend kernel's resident threads -- always the
    // case here, the image being at most TRACER_NOALLOC_MAX_PIXELS), the
    // finishing kernel traces every pixel in one launch; otherwise every round
    // is launched, and a round with an empty queue returns at once.
    const uint32_t no_rounds_below = p->tail_paths ? p->tail_paths : wc.extend_grid * wc.block;
    const int fin_per = npx < no_rounds_below ? wf_finish_blocks_per_sm(wc, stack) : 0;
    if (fin_per > 0) {
        const size_t blocks = (npx + 127) / 128, cap = (size_t)fin_per * c->sm_count;
        wc.finish_grid = (uint32_t)(blocks < cap ? blocks : cap);
        if (e == cudaSuccess) e = wf_launch_finish(a, ws, wc, 0, st);
    } else {
        const uint32_t rounds = p->spp * p->max_depth + 1;
        for (uint32_t k = 0; k < rounds && e == cudaSuccess; ++k) {
            e = wf_launch_extend(a, ws, wc, (int)(k & 1), st);
            if (e == cudaSuccess) e = wf_launch_shade(a, ws, wc, (int)(k & 1), st);
        }
    }
    if (e != cudaSuccess) return cuda_fail(c, e, "no-alloc trace launch");
    return TRACER_OK;
}

// ------------------------------------------------------------------ batches
namespace {

// One scene packed for the device: triangles in leaf order as (v0, material)
// (v1 - v0, id) (v2 - v0, 0), sphere centres/radii in leaf order, BVH nodes.
struct PackedScene {
    std::vector<float4> tri, geo;
    std::vector<uint32_t> sid, emit;
    std::vector<tracer_bvh_node> tnodes, snodes, tenc, senc;
    std::vector<WideNode> twide, swide;
    std::vector<Cw8Node> cw8;
    std::vector<float4> cw8_prims;
    uint32_t depth = 0, wide_depth = 0, cw8_depth = 0;
    bool wide = false, cw8_ok = false;
    int status = TRACER_OK;
};

void pack_scene(const tracer_scene_desc& d, PackedScene& out)
{
    std::vector<uint32_t> tidx, sidx;
    uint32_t td = 0, sd = 0;
    if (d.num_triangles) {
        if (d.tri_nodes) {
            out.status = tracer_validate_bvh(TRACER_PRIM_TRIANGLE, d.triangles, d.num_triangles, d.tri_nodes,
                                             d.num_tri_nodes, d.tri_prim_index, &td);
            if (out.status != TRACER_OK) return;
            out.tnodes.assign(d.tri_nodes, d.tri_nodes + d.num_tri_nodes);
            tidx.assign(d.tri_prim_index, d.tri_prim_index + d.num_triangles);
        } else {
            out.tnodes.resize(2 * (size_t)d.num_triangles);
            tidx.resize(d.num_triangles);
            uint32_t nn = 0;
            out.status = tracer_build_bvh(d.bvh, TRACER_PRIM_TRIANGLE, d.triangles, d.num_triangles, d.leaf_size,
                                          d.sah_bins, out.tnodes.data(), &nn, tidx.data(), &td);
            if (out.status != TRACER_OK) return;
            out.tnodes.resize(nn);
        }
    }
    if (d.num_spheres) {
        if (d.sphere_nodes) {
            out.status = tracer_validate_bvh(TRACER_PRIM_SPHERE, d.spheres, d.num_spheres, d.sphere_nodes,
                                             d.num_sphere_nodes, d.sphere_prim_index, &sd);
            if (out.status != TRACER_OK) return;
            out.snodes.assign(d.sphere_nodes, d.sphere_nodes + d.num_sphere_nodes);
            sidx.assign(d.sphere_prim_index, d.sphere_prim_index + d.num_spheres);
        } else {
            out.snodes.resize(2 * (size_t)d.num_spheres);
            sidx.resize(d.num_spheres);
            uint32_t nn = 0;
            out.status = tracer_build_bvh(d.bvh, TRACER_PRIM_SPHERE, d.spheres, d.num_spheres, d.leaf_size,
                                          d.sah_bins, out.snodes.data(), &nn, sidx.data(), &sd);
            if (out.status != TRACER_OK) return;
            out.snodes.resize(nn);
        }
    }
    out.depth = td > sd ? td : sd;
    uint32_t twd = 0, swd = 0;
    out.wide = collapse_wide4(out.tnodes.data(), (uint32_t)out.tnodes.size(), out.twide, &twd) &&
               collapse_wide4(out.snodes.data(), (uint32_t)out.snodes.size(), out.swide, &swd);
    out.wide_depth = twd > swd ? twd : swd;
    if (!encode_refs(out.tnodes.data(), (uint32_t)out.tnodes.size(), out.tenc) ||
        !encode_refs(out.snodes.data(), (uint32_t)out.snodes.size(), out.senc)) {
        out.status = TRACER_ERR_BAD_BVH;
        return;
    }
    out.tri.resize(3 * (size_t)d.num_triangles);
    for (uint32_t k = 0; k < d.num_triangles; ++k) {
        const uint32_t i = tidx[k];
        const tracer_triangle& t = d.triangles[i];
        float m, id;
        std::memcpy(&m, &t.material, 4);
        std::memcpy(&id, &i, 4);
        out.tri[3 * k + 0] = make_float4(t.v0[0], t.v0[1], t.v0[2], m);
        out.tri[3 * k + 1] = make_float4(t.v1[0] - t.v0[0], t.v1[1] - t.v0[1], t.v1[2] - t.v0[2], id);
        out.tri[3 * k + 2] = make_float4(t.v2[0] - t.v0[0], t.v2[1] - t.v0[1], t.v2[2] - t.v0[2], 0.0f);
    }
    out.geo.resize(d.num_spheres);
    out.sid.resize(d.num_spheres);
    for (uint32_t k = 0; k < d.num_spheres; ++k) {
        const uint32_t i = sidx[k];
        const tracer_sphere& q = d.spheres[i];
        out.geo[k] = make_float4(q.P[0], q.P[1], q.P[2], q.r);
        out.sid[k] = i;
    }
    for (uint32_t i = 0; i < d.num_spheres; ++i) {
        const float* em = d.spheres[i].mat.emissive;
        if (!(em[0] == 0.0f && em[1] == 0.0f && em[2] == 0.0f)) out.emit.push_back(i);
    }
    out.cw8_ok = d.num_triangles > 0 && d.num_spheres == 0 &&
                 make_cw8(out.tnodes, out.tri, out.cw8, out.cw8_prims, out.cw8_depth);
}

int validate_desc(tracer_ctx* c, const tracer_scene_desc& d, uint32_t k)
{
    if ((d.num_triangles && !d.triangles) || (d.num_spheres && !d.spheres) || (d.num_planes && !d.planes) ||
        (d.num_materials && !d.materials))
        return fail(c, TRACER_ERR_INVALID_ARG, "scene %u: null array with a nonzero count", k);
    if (d.bvh != TRACER_BVH_MEDIAN && d.bvh != TRACER_BVH_SAH)
        return fail(c, TRACER_ERR_INVALID_ARG, "scene %u: batches need a BVH (median or SAH)", k);
    if ((uint64_t)d.num_triangles + d.num_spheres + d.num_planes >= 0xFFFFFFFFull)
        return fail(c, TRACER_ERR_INVALID_ARG, "scene %u: too many primitives", k);
    for (uint32_t i = 0; i < d.num_triangles; ++i)
        if (d.triangles[i].material >= d.num_materials)
            return fail(c, TRACER_ERR_INVALID_ARG, "scene %u: triangle %u uses material %u of %u", k, i,
                        d.triangles[i].material, d.num_materials);
    return TRACER_OK;
}

}  // namespace

extern "C" int tracer_upload_scenes(tracer_ctx* c, const tracer_scene_desc* descs, uint32_t n)
{
    if (!c) return TRACER_ERR_INVALID_ARG;
    if (!descs || n == 0) return fail(c, TRACER_ERR_INVALID_ARG, "empty batch");
    for (uint32_t k = 0; k < n; ++k) {
        int r = validate_desc(c, descs[k], k);
        if (r != TRACER_OK) return r;
    }
    int r = finish(c);
    if (r != TRACER_OK) return r;
    cudaSetDevice(c->device);
    // BVH builds in parallel on host threads (each scene is independent)
    std::vector<PackedScene> packed(n);
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const unsigned nt = std::min<unsigned>(hw, n);
    std::vector<std::thread> pool;
    std::atomic<uint32_t> next{0};
    for (unsigned t = 0; t < nt; ++t)
        pool.emplace_back([&]() {
            for (uint32_t k = next++; k < n; k = next++) pack_scene(descs[k], packed[k]);
        });
    for (auto& th : pool) th.join();
    for (uint32_t k = 0; k < n; ++k)
        if (packed[k].status != TRACER_OK)
            return fail(c, packed[k].status, "scene %u: BVH build or validation failed", k);

    // one arena per array kind, scenes back to back
    std::vector<float4> tri, mats, geo, rec, planes, tnodes, snodes, twide, swide, tenc, senc, tcw8, tcw8p;
    std::vector<uint32_t> sid, emit;
    struct Off {
        size_t tri, mats, geo, rec, planes, tnodes, snodes, sid, emit, twide, swide, tenc, senc, tcw8, tcw8p;
    };
    std::vector<Off> off(n);
    bool wide_all = true, cw8_all = true;
    for (uint32_t k = 0; k < n; ++k)
        cw8_all = cw8_all && packed[k].cw8_ok;
    for (uint32_t k = 0; k < n; ++k) {
        const tracer_scene_desc& d = descs[k];
        const PackedScene& p = packed[k];
        off[k] = Off{tri.size(),    mats.size(),  geo.size(),  rec.size(),  planes.size(),
                     tnodes.size(), snodes.size(), sid.size(), emit.size(), twide.size(),
                     swide.size(),  tenc.size(),  senc.size(), tcw8.size(), tcw8p.size()};
        if (cw8_all) {  // 6 and 4 float4 per record: every scene's part stays 32-byte aligned
            const float4* cn = reinterpret_cast<const float4*>(p.cw8.data());
            tcw8.insert(tcw8.end(), cn, cn + 6 * p.cw8.size());
            tcw8p.insert(tcw8p.end(), p.cw8_prims.begin(), p.cw8_prims.end());
        }
        const float4* te = reinterpret_cast<const float4*>(p.tenc.data());
        tenc.insert(tenc.end(), te, te + 2 * p.tenc.size());
        const float4* se = reinterpret_cast<const float4*>(p.senc.data());
        senc.insert(senc.end(), se, se + 2 * p.senc.size());
        wide_all = wide_all && p.wide;
        const float4* tw = reinterpret_cast<const float4*>(p.twide.data());
        twide.insert(twide.end(), tw, tw + 8 * p.twide.size());
        const float4* sw = reinterpret_cast<const float4*>(p.swide.data());
        swide.insert(swide.end(), sw, sw + 8 * p.swide.size());
        tri.insert(tri.end(), p.tri.begin(), p.tri.end());
        const float4* m = reinterpret_cast<const float4*>(d.materials);
        mats.insert(mats.end(), m, m + 3 * (size_t)d.num_materials);
        geo.insert(geo.end(), p.geo.begin(), p.geo.end());
        const float4* sr = reinterpret_cast<const float4*>(d.spheres);
        rec.insert(rec.end(), sr, sr + 4 * (size_t)d.num_spheres);
        const float4* pl = reinterpret_cast<const float4*>(d.planes);
        planes.insert(planes.end(), pl, pl + 4 * (size_t)d.num_planes);
        const float4* tn = reinterpret_cast<const float4*>(p.tnodes.data());
        tnodes.insert(tnodes.end(), tn, tn + 2 * p.tnodes.size());
        const float4* sn = reinterpret_cast<const float4*>(p.snodes.data());
        snodes.insert(snodes.end(), sn, sn + 2 * p.snodes.size());
        sid.insert(sid.end(), p.sid.begin(), p.sid.end());
        emit.insert(emit.end(), p.emit.begin(), p.emit.end());
    }
    SceneBuffers& b = c->batch;
    b.release();
    cudaError_t e = upload(b.tri, tri.data(), tri.size());
    if (e == cudaSuccess) e = upload(b.mats, mats.data(), mats.size());
    if (e == cudaSuccess) e = upload(b.sph_geo, geo.data(), geo.size());
    if (e == cudaSuccess) e = upload(b.sph_rec, rec.data(), rec.size());
    if (e == cudaSuccess) e = upload(b.planes, planes.data(), planes.size());
    if (e == cudaSuccess) e = upload(b.tri_nodes, tnodes.data(), tnodes.size());
    if (e == cudaSuccess) e = upload(b.sph_nodes, snodes.data(), snodes.size());
    if (e == cudaSuccess) e = upload(b.sph_id, sid.data(), sid.size());
    if (e == cudaSuccess) e = upload(b.emit, emit.data(), emit.size());
    if (e == cudaSuccess) e = upload(b.tri_enc, tenc.data(), tenc.size());
    if (e == cudaSuccess) e = upload(b.sph_enc, senc.data(), senc.size());
    if (e == cudaSuccess && wide_all) e = upload(b.tri_wide, twide.data(), twide.size());
    if (e == cudaSuccess && wide_all) e = upload(b.sph_wide, swide.data(), swide.size());
    if (e == cudaSuccess && cw8_all) e = upload(b.tri_cw8, tcw8.data(), tcw8.size());
    if (e == cudaSuccess && cw8_all) e = upload(b.tri_cw8_prims, tcw8p.data(), tcw8p.size());
    if (e != cudaSuccess) {
        b.release();
        return cuda_fail(c, e, "batch upload");
    }
    b.wide = wide_all;
    b.wide_depth = 0;
    b.cw8 = cw8_all;
    b.cw8_depth = 0;
    c->batch_scenes.assign(n, DevScene{});
    c->batch_depth.assign(n, 0);
    c->batch_nodes.assign(n, 0);
    c->batch_emitters = false;
    for (uint32_t k = 0; k < n; ++k) {
        const tracer_scene_desc& d = descs[k];
        const PackedScene& p = packed[k];
        auto at = [](auto& buf, size_t o) { return buf.p ? buf.p + o : nullptr; };
        c->batch_scenes[k] = DevScene{at(b.tri, off[k].tri), at(b.mats, off[k].mats), at(b.sph_geo, off[k].geo),
                                      at(b.sph_id, off[k].sid), at(b.sph_rec, off[k].rec), at(b.planes, off[k].planes),
                                      at(b.emit, off[k].emit), at(b.tri_nodes, off[k].tnodes),
                                      at(b.sph_nodes, off[k].snodes), d.num_triangles, d.num_materials, d.num_spheres,
                                      d.num_planes, (uint32_t)p.emit.size(), (uint32_t)p.tnodes.size(),
                                      (uint32_t)p.snodes.size(),
                                      wide_all ? at(b.tri_wide, off[k].twide) : nullptr,
                                      wide_all ? at(b.sph_wide, off[k].swide) : nullptr,
                                      at(b.tri_enc, off[k].tenc), at(b.sph_enc, off[k].senc),
                                      cw8_all ? at(b.tri_cw8, off[k].tcw8) : nullptr,
                                      cw8_all ? at(b.tri_cw8_prims, off[k].tcw8p) : nullptr};
        b.wide_depth = std::max(b.wide_depth, p.wide_depth);
        b.cw8_depth = std::max(b.cw8_depth, p.cw8_depth);
        c->batch_depth[k] = p.depth;
        c->batch_nodes[k] = (uint32_t)std::max(p.tnodes.size(), p.snodes.size());
        c->batch_emitters = c->batch_emitters || !p.emit.empty();
    }
    b.nt = (uint32_t)(tri.size() / 3);
    b.bvh = true;
    b.loaded = true;
    c->graph_key.clear();
    return TRACER_OK;
}

extern "C" int tracer_trace_batched(tracer_ctx* c, const tracer_frame* frames, const tracer_trace_params* params,
                                    uint32_t n, int use_graph, void* cuda_stream)
{
    if (!c) return TRACER_ERR_INVALID_ARG;
    if (!frames || !params) return fail(c, TRACER_ERR_INVALID_ARG, "null frames or params");
    if (!c->batch.loaded) return fail(c, TRACER_ERR_NO_SCENE, "no batch uploaded");
    if (n != c->batch_scenes.size())
        return fail(c, TRACER_ERR_INVALID_ARG, "batch holds %zu scenes, %u given", c->batch_scenes.size(), n);
    const tracer_trace_params& p0 = params[0];
    const int kernel = p0.kernel == TRACER_KERNEL_AUTO ? TRACER_KERNEL_WAVEFRONT : p0.kernel;
    if (kernel != TRACER_KERNEL_PLAIN && kernel != TRACER_KERNEL_WAVEFRONT)
        return fail(c, TRACER_ERR_INVALID_ARG, "unknown kernel %d", p0.kernel);
    const uint32_t block = p0.block ? p0.block : 128;
    if (kernel == TRACER_KERNEL_WAVEFRONT && block != 64 && block != 128 && block != 256)
        return fail(c, TRACER_ERR_INVALID_ARG, "wavefront block must be 64, 128 or 256");
    if (kernel == TRACER_KERNEL_PLAIN && (block % 32 != 0 || block < 32 || block > 256))
        return fail(c, TRACER_ERR_INVALID_ARG, "block %u must be a multiple of 32 in [32, 256]", block);
    uint32_t need = 1, max_nodes = 0;
    for (uint32_t k = 0; k < n; ++k) {
        need = std::max(need, c->batch_depth[k]);
        max_nodes = std::max(max_nodes, c->batch_nodes[k]);
    }
    uint32_t stack = p0.stack_depth ? p0.stack_depth : need;
    if (stack < need) return fail(c, TRACER_ERR_STACK_OVERFLOW, "stack depth %u below the BVH depth %u", stack, need);
    if ((size_t)stack * 256 * 8 > 200 * 1024)
        return fail(c, TRACER_ERR_INVALID_ARG, "stack depth %u exceeds shared memory", stack);
    int wide = 0;
    if (kernel == TRACER_KERNEL_WAVEFRONT) {
        int rw = pick_width_for(c, &p0, c->batch.wide, c->batch.wide_depth, c->batch.cw8, c->batch.cw8_depth, stack,
                                wide);
        if (rw != TRACER_OK) return rw;
    }
    const uint32_t mask = p0.aov_mask ? p0.aov_mask : (1u << TRACER_AOV_RGBA8);
    const int stats = (p0.stats || (mask & (1u << TRACER_AOV_STATS))) ? 1 : 0;
    std::vector<size_t> base(n);
    size_t total = 0;
    uint64_t max_rounds = 0;
    for (uint32_t k = 0; k < n; ++k) {
        const tracer_trace_params& p = params[k];
        if (p.width == 0 || p.height == 0 || p.width > 32768 || p.height > 32768)
            return fail(c, TRACER_ERR_NO_SUITABLE_SURFACE, "scene %u: image size %ux%u", k, p.width, p.height);
        if (p.spp == 0 || p.max_depth == 0 || p.max_depth > 1024 || p.spp > 1u << 20)
            return fail(c, TRACER_ERR_INVALID_ARG, "scene %u: spp / max_depth out of range", k);
        if (p.tie_mode != TRACER_TIES_STRICT) return fail(c, TRACER_ERR_INVALID_ARG, "batches use strict ties");
        base[k] = total;
        total += (size_t)p.width * p.height;
        max_rounds = std::max<uint64_t>(max_rounds, (uint64_t)p.spp * p.max_depth + 1);
    }
    if (total >= 0xFFFFFFFFull) return fail(c, TRACER_ERR_NO_SUITABLE_SURFACE, "batch has too many pixels");
    int r = finish(c);
    if (r != TRACER_OK) return r;
    cudaSetDevice(c->device);
    cudaError_t e = cudaSuccess;
    if (mask & (1u << TRACER_AOV_RGBA8)) e = dalloc(c->b_rgba8, total);
    if (e == cudaSuccess && (mask & (1u << TRACER_AOV_RGBA32F))) e = dalloc(c->b_rgba32f, total);
    if (e == cudaSuccess && (mask & (1u << TRACER_AOV_PRIMARY_HIT))) e = dalloc(c->b_hit, total);
    if (e == cudaSuccess) e = dalloc(c->batch_slots, n);
    if (e == cudaSuccess && c->pinned_slots_n < n) {
        if (c->pinned_slots) cudaFreeHost(c->pinned_slots);
        c->pinned_slots = nullptr;
        c->pinned_slots_n = 0;
        e = cudaMallocHost(&c->pinned_slots, sizeof(TraceArgs) * n);
        if (e == cudaSuccess) c->pinned_slots_n = n;
    }
    if (e == cudaSuccess && kernel == TRACER_KERNEL_WAVEFRONT) {
        e = ensure_wavefront(c, total);
        if (e == cudaSuccess) e = dalloc(c->wf_scene, total);
    }
    if (e != cudaSuccess) return cuda_fail(c, e, "batch allocation");
    c->b_mask = mask | (stats ? (1u << TRACER_AOV_STATS) : 0u);
    c->batch_base = base;
    c->batch_w.resize(n);
    c->batch_h.resize(n);

    cudaStream_t st = cuda_stream ? static_cast<cudaStream_t>(cuda_stream) : c->stream;
    // per-scene arguments, written to pinned memory and copied to the table
    // (stream-ordered after the previous trace that read it)
    TraceArgs* slots = c->pinned_slots;
    for (uint32_t k = 0; k < n; ++k) {
        const tracer_trace_params& p = params[k];
        const tracer_frame& f = frames[k];
        TraceArgs& a = slots[k];
        std::memset(&a, 0, sizeof a);
        a.sc = c->batch_scenes[k];
        if (wide != WF_WIDTH_8) a.sc.tri_cw8 = a.sc.tri_cw8_prims = nullptr;  // finishing kernel: binary too
        a.fr.aspect = f.aspect_ratio;
        a.fr.seed = f.seed;
        a.fr.cpos = V3{f.camera.pos[0], f.camera.pos[1], f.camera.pos[2]};
        a.fr.cdir = V3{f.camera.dir[0], f.camera.dir[1], f.camera.dir[2]};
        a.fr.cright = V3{f.camera.right[0], f.camera.right[1], f.camera.right[2]};
        a.fr.cup = V3{f.camera.up[0], f.camera.up[1], f.camera.up[2]};
        a.width = p.width;
        a.height = p.height;
        a.spp = p.spp;
        a.max_depth = p.max_depth;
        a.rr_start = p.rr_start;
        a.sky = V3{p.sky[0], p.sky[1], p.sky[2]};
        a.sky_on = !(p.sky[0] == 0.0f && p.sky[1] == 0.0f && p.sky[2] == 0.0f);
        a.stack_depth = stack;
        a.trav_limit = trav_limit(c, c->batch_nodes[k]);
        a.rgba8 = (mask & (1u << TRACER_AOV_RGBA8)) ? c->b_rgba8.p + base[k] : nullptr;
        a.rgba32f = (mask & (1u << TRACER_AOV_RGBA32F)) ? c->b_rgba32f.p + base[k] : nullptr;
        a.hit = (mask & (1u << TRACER_AOV_PRIMARY_HIT)) ? c->b_hit.p + base[k] : nullptr;
        a.stats = c->stats.p;
        a.status = c->status.p;
        a.pixel_base = (uint32_t)base[k];
        a.num_slots = (uint32_t)total;
        c->batch_w[k] = p.width;
        c->batch_h[k] = p.height;
    }
    e = cudaMemcpyAsync(c->batch_slots.p, slots, sizeof(TraceArgs) * n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->stats.p, 0, sizeof(unsigned long long) * C_COUNT, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->status.p, 0, sizeof(int), st);
    if (e != cudaSuccess) return cuda_fail(c, e, "batch set-up");
    c->last_kernel = kernel;
    c->last_rounds = 0;
    c->last_prof_rounds = 0;
    c->last_round_entries = 0;
    c->last_finish = false;
    c->last_launches = 0;
    if (c->profiling) cudaEventRecord(c->prof_begin, st);

    if (kernel == TRACER_KERNEL_PLAIN) {
        LaunchConfig lc{block, stats, TRACER_TIES_STRICT, 1};
        for (uint32_t k = 0; k < n && e == cudaSuccess; ++k) {
            e = launch_plain(slots[k], lc, st);
            c->last_launches++;
        }
    } else {
        TraceArgs a = slots[0];
        a.num_slots = (uint32_t)total;
        a.stack_depth = stack;
        a.trav_limit = trav_limit(c, max_nodes);
        WfConfig wc;
        std::memset(&wc, 0, sizeof wc);
        wc.tie = TRACER_TIES_STRICT;
        wc.bvh = 1;
        wc.stats = stats;
        wc.multi = 1;
        wc.has_emitters = c->batch_emitters;
        wc.block = block;
        wc.wide = wide;
        if (wide == WF_WIDTH_8) wc.cw8_stack = c->batch.cw8_depth;
        wc.slots = c->batch_slots.p;
        wc.nslots = n;
        if (!use_graph) {
            r = run_wavefront(c, a, wc, total, max_rounds, stack, p0.wavefront, p0.tail_paths, st);
            if (r != TRACER_OK) return r;
        } else {
            WfState ws{c->wf_ray_o.p, c->wf_ray_d.p, c->wf_hit.p, c->wf_acc.p, c->wf_mask.p, c->wf_accum.p,
                       c->wf_prim0.p, {c->wf_q0.p, c->wf_q1.p}, c->wf_count.p, c->wf_scene.p};
            int per = wf_extend_blocks_per_sm(wc, stack);
            if (per <= 0) return fail(c, TRACER_ERR_INVALID_ARG, "extend kernel cannot be resident");
            if (p0.wavefront && (int)p0.wavefront < per) per = (int)p0.wavefront;
            wc.extend_grid = (uint32_t)(per * c->sm_count);
            const size_t sg = (total + 255) / 256;
            wc.shade_grid = (uint32_t)(sg < (size_t)c->sm_count * 8 ? sg : (size_t)c->sm_count * 8);
            // the graph bakes in sizes, launch shapes and buffer addresses
            std::vector<uint64_t> key = {n, total, max_rounds, block, stack, (uint64_t)stats, wc.extend_grid,
                                         (uint64_t)wide, p0.tail_paths,
                                         (uint64_t)(uintptr_t)c->wf_ray_o.p, (uint64_t)(uintptr_t)c->batch_slots.p,
                                         (uint64_t)(uintptr_t)c->b_rgba8.p, (uint64_t)(uintptr_t)c->b_rgba32f.p,
                                         (uint64_t)(uintptr_t)c->b_hit.p, mask};
            if (key != c->graph_key || !c->graph_exec) {
                if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
                if (c->graph) cudaGraphDestroy(c->graph);
                c->graph_exec = nullptr;
                c->graph = nullptr;
                c->graph_key.clear();
                // The graph has no queue lengths to look at, so the round at
                // which the finishing kernel takes over is the one a traced
                // run of this batch reaches (launched here, with read-backs).
                // Any frame is still traced completely: the finishing kernel
                // runs whatever paths are queued after that round.
                r = run_wavefront(c, a, wc, total, max_rounds, stack, p0.wavefront, p0.tail_paths, st);
                if (r != TRACER_OK) return r;
                const int fin_per = c->last_finish ? wf_finish_blocks_per_sm(wc, stack) : 0;
                const uint64_t rounds = fin_per > 0 ? c->last_handover : max_rounds;
                c->graph_rounds = rounds;
                c->graph_finish = fin_per > 0;
                cudaStream_t cap;
                e = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking);
                if (e != cudaSuccess) return cuda_fail(c, e, "graph capture stream");
                e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
                if (e == cudaSuccess) e = wf_launch_generate(a, ws, wc, cap);
                for (uint64_t k = 0; k < rounds && e == cudaSuccess; ++k) {
                    e = wf_launch_extend(a, ws, wc, (int)(k & 1), cap);
                    if (e == cudaSuccess) e = wf_launch_shade(a, ws, wc, (int)(k & 1), cap);
                }
                if (e == cudaSuccess && fin_per > 0) {
                    wc.finish_grid = (uint32_t)(fin_per * c->sm_count);
                    e = wf_launch_finish(a, ws, wc, (int)(rounds & 1), cap);
                }
                cudaGraph_t g = nullptr;
                cudaError_t e2 = cudaStreamEndCapture(cap, &g);
                if (e == cudaSuccess) e = e2;
                if (e == cudaSuccess) e = cudaGraphInstantiate(&c->graph_exec, g, 0);
                cudaStreamDestroy(cap);
                if (e != cudaSuccess) {
                    if (g) cudaGraphDestroy(g);
                    return cuda_fail(c, e, "graph capture");
                }
                c->graph = g;
                c->graph_key = key;
            }
            e = cudaGraphLaunch(c->graph_exec, st);
            c->last_rounds = (uint32_t)c->graph_rounds;
            c->last_launches = (uint32_t)(1 + 2 * c->graph_rounds + (c->graph_finish ? 1 : 0));
            c->last_finish = c->graph_finish;
            c->last_prof_rounds = 0;  // the graph's rounds are not timed one by one
            c->last_round_entries = 0;
        }
    }
    if (c->profiling) cudaEventRecord(c->prof_end, st);
    if (e == cudaSuccess) e = cudaEventRecord(c->done, st);
    if (e != cudaSuccess) return cuda_fail(c, e, "batched trace launch");
    c->pending = true;
    return TRACER_OK;
}

extern "C" int tracer_readback_scene(tracer_ctx* c, uint32_t scene, int aov, void* dst, size_t bytes)
{
    if (!c) return TRACER_ERR_INVALID_ARG;
    if (!dst) return fail(c, TRACER_ERR_INVALID_ARG, "null destination");
    if (scene >= c->batch_w.size()) return fail(c, TRACER_ERR_INVALID_ARG, "scene %u not in the last batch", scene);
    cudaSetDevice(c->device);
    int r = finish(c);
    if (r != TRACER_OK) return r;
    const uint32_t bit = aov >= 0 && aov < 32 ? (1u << aov) : 0;
    if (!bit || !(c->b_mask & bit))
        return fail(c, TRACER_ERR_NO_SUITABLE_SURFACE, "AOV %d was not produced by the last batch", aov);
    const size_t npx = (size_t)c->batch_w[scene] * c->batch_h[scene];
    const size_t b = c->batch_base[scene];
    const void* src;
    size_t n;
    switch (aov) {
    case TRACER_AOV_RGBA8: src = c->b_rgba8.p + b; n = npx * 4; break;
    case TRACER_AOV_RGBA32F: src = c->b_rgba32f.p + b; n = npx * 16; break;
    case TRACER_AOV_PRIMARY_HIT: src = c->b_hit.p + b; n = npx * 8; break;
    case TRACER_AOV_STATS: src = c->stats.p; n = sizeof(tracer_stats); break;
    default: return fail(c, TRACER_ERR_NO_SUITABLE_SURFACE, "unknown AOV %d", aov);
    }
    if (bytes != n) return fail(c, TRACER_ERR_INVALID_ARG, "AOV %d of scene %u holds %zu bytes, %zu requested", aov,
                                scene, n, bytes);
    cudaError_t e = cudaMemcpy(dst, src, n, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(c, e, "readback");
    return TRACER_OK;
}

// ------------------------------------------------------------------ adjoint
namespace {

bool is_device_ptr(const void* p)
{
    if (!p) return false;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();  // an unregistered host pointer is not an error
        return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}


}  // namespace

extern "C" int tracer_trace_adjoint(tracer_ctx* c, const tracer_frame* f, const tracer_trace_params* p,
                                    const float* dL_dimage, const float* linear_image, float* d_albedo,
                                    float* d_emission, float* d_campos, void* cuda_stream)
{
    if (!c) return TRACER_ERR_INVALID_ARG;
    if (!f || !p || !dL_dimage) return fail(c, TRACER_ERR_INVALID_ARG, "null frame, params or dL/dI");
    if (!c->scene.loaded) return fail(c, TRACER_ERR_NO_SCENE, "no scene uploaded");
    if (p->width == 0 || p->height == 0 || p->width > 32768 || p->height > 32768)
        return fail(c, TRACER_ERR_NO_SUITABLE_SURFACE, "image size %ux%u not supported", p->width, p->height);
    if (p->spp == 0 || p->max_depth == 0 || p->max_depth > 1024 || p->spp > 1u << 20)
        return fail(c, TRACER_ERR_INVALID_ARG, "spp %u / max_depth %u out of range", p->spp, p->max_depth);
    if (p->tie_mode != TRACER_TIES_REFERENCE && p->tie_mode != TRACER_TIES_STRICT)
        return fail(c, TRACER_ERR_INVALID_ARG, "unknown tie mode %d", p->tie_mode);
    if (p->tie_mode == TRACER_TIES_REFERENCE && c->scene.bvh)
        return fail(c, TRACER_ERR_INVALID_ARG, "reference ties depend on scan order and need a linear-scan scene");
    const SceneBuffers& s = c->scene;
    const uint32_t need = s.bvh ? (s.depth > 1 ? s.depth : 1) : 0;
    const uint32_t stack = p->stack_depth ? p->stack_depth : need;
    if (s.bvh && stack < need)
        return fail(c, TRACER_ERR_STACK_OVERFLOW, "stack depth %u below the BVH depth %u", stack, need);
    if ((size_t)stack * 128 * 8 > 100 * 1024)
        return fail(c, TRACER_ERR_INVALID_ARG, "stack depth %u exceeds shared memory", stack);
    // AUTO: the wavefront wherever it applies (below).  With its finishing
    // kernel it is the faster form at every size measured on the c3 scene
    // (per-pixel / wavefront ms): 64^2 x 4 spp 1.29 / 1.25, 128^2 1.30 / 1.13,
    // 256^2 1.72 / 1.36, 512^2 4.65 / 2.48; 1024^2 x 64 spp: 5.8x.
    const int kernel = p->kernel == TRACER_KERNEL_AUTO ? TRACER_KERNEL_WAVEFRONT : p->kernel;
    if (kernel != TRACER_KERNEL_PLAIN && kernel != TRACER_KERNEL_WAVEFRONT)
        return fail(c, TRACER_ERR_INVALID_ARG, "unknown kernel %d", p->kernel);
    const uint32_t wblock = p->block ? p->block : 128;
    if (kernel == TRACER_KERNEL_WAVEFRONT && wblock != 64 && wblock != 128 && wblock != 256)
        return fail(c, TRACER_ERR_INVALID_ARG, "wavefront block must be 64, 128 or 256");
    // The wavefront form covers scenes without emissive spheres (no next-event
    // estimation, zero camera gradient) given the forward linear image; the
    // per-pixel kernel covers everything.
    const bool use_wf = kernel == TRACER_KERNEL_WAVEFRONT && s.ne == 0 && linear_image != nullptr &&
                        p->max_depth <= 1000 && p->spp < 32768u;
    int r = finish(c);
    if (r != TRACER_OK) return r;
    cudaSetDevice(c->device);
    AdjBuffers& ab = c->adj;
    const size_t npx = (size_t)p->width * p->height;
    const size_t ng = 6 * (size_t)s.nm + 3;
    cudaStream_t st = cuda_stream ? static_cast<cudaStream_t>(cuda_stream) : c->stream;
    cudaError_t e = dalloc(ab.grad, ng);
    if (e == cudaSuccess) e = dalloc(ab.gradf, ng);
    const float4* dldi = reinterpret_cast<const float4*>(dL_dimage);
    if (e == cudaSuccess && !is_device_ptr(dL_dimage)) {
        e = dalloc(ab.dldi, npx);
        if (e == cudaSuccess) e = cudaMemcpyAsync(ab.dldi.p, dL_dimage, npx * 16, cudaMemcpyHostToDevice, st);
        dldi = ab.dldi.p;
    }
    const float4* lin = reinterpret_cast<const float4*>(linear_image);
    if (e == cudaSuccess && linear_image && !is_device_ptr(linear_image)) {
        e = dalloc(ab.lin, npx);
        if (e == cudaSuccess) e = cudaMemcpyAsync(ab.lin.p, linear_image, npx * 16, cudaMemcpyHostToDevice, st);
        lin = ab.lin.p;
    }
    // the boundary term's list of visible outline parts: room for 16 per edge
    // piece on average (c3: 640k parts, 31 MB); parts beyond it are
    // evaluated by the walk itself
    const bool edges = d_campos && s.nt > 0 && c->edge_samples > 0;
    uint32_t seg_cap = 0;
    if (edges) {
        const uint64_t cap64 = std::min<uint64_t>(16ull * s.nt * 3u * c->edge_samples, 1ull << 25);
        seg_cap = (uint32_t)std::max<uint64_t>(cap64, 1u << 16);
        if (e == cudaSuccess) e = dalloc(ab.segs, 3 * (size_t)seg_cap);
        if (e == cudaSuccess) e = dalloc(ab.nsegs, 1);
        if (e == cudaSuccess) e = cudaMemsetAsync(ab.nsegs.p, 0, sizeof(uint32_t), st);
    }
    if (e == cudaSuccess) e = cudaMemsetAsync(ab.grad.p, 0, ng * sizeof(double), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->stats.p, 0, sizeof(unsigned long long) * C_COUNT, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->status.p, 0, sizeof(int), st);
    if (e != cudaSuccess) return cuda_fail(c, e, "adjoint set-up");

    TraceArgs a;
    std::memset(&a, 0, sizeof a);
    a.sc = DevScene{s.tri.p, s.mats.p, s.sph_geo.p, s.sph_id.p, s.sph_rec.p, s.planes.p, s.emit.p, s.tri_nodes.p,
                    s.sph_nodes.p, s.nt, s.nm, s.ns, s.np, s.ne, s.n_tri_nodes, s.n_sph_nodes,
                    s.tri_wide.p, s.sph_wide.p, s.tri_enc.p, s.sph_enc.p, s.tri_cw8.p, s.tri_cw8_prims.p};
    a.fr.aspect = f->aspect_ratio;
    a.fr.seed = f->seed;
    a.fr.cpos = V3{f->camera.pos[0], f->camera.pos[1], f->camera.pos[2]};
    a.fr.cdir = V3{f->camera.dir[0], f->camera.dir[1], f->camera.dir[2]};
    a.fr.cright = V3{f->camera.right[0], f->camera.right[1], f->camera.right[2]};
    a.fr.cup = V3{f->camera.up[0], f->camera.up[1], f->camera.up[2]};
    a.width = p->width;
    a.height = p->height;
    a.spp = p->spp;
    a.max_depth = p->max_depth;
    a.rr_start = p->rr_start;
    a.sky = V3{p->sky[0], p->sky[1], p->sky[2]};
    a.sky_on = !(p->sky[0] == 0.0f && p->sky[1] == 0.0f && p->sky[2] == 0.0f);
    a.stack_depth = stack;
    const uint32_t nn = s.n_tri_nodes > s.n_sph_nodes ? s.n_tri_nodes : s.n_sph_nodes;
    a.trav_limit = trav_limit(c, nn);
    a.stats = c->stats.p;
    a.status = c->status.p;
    c->last_rounds = 0;
    c->last_prof_rounds = 0;
    c->last_round_entries = 0;
    c->last_finish = false;
    c->last_mask = 1u << TRACER_AOV_STATS;
    c->width = p->width;
    c->height = p->height;
    if (use_wf) {
        e = ensure_wavefront(c, npx);
        if (e == cudaSuccess) e = dalloc(ab.pix, npx);
        // pass 1's hits for pass 2 to replay without tracing, when they fit the limit
        const size_t log_n = npx * (size_t)p->max_depth;
        const bool use_log = log_n * sizeof(uint4) <= c->adj_log_limit;
        if (e == cudaSuccess && use_log) e = dalloc(ab.log, log_n);
        if (e != cudaSuccess) return cuda_fail(c, e, "wavefront adjoint state allocation");
        a.pixel_base = 0;
        a.num_slots = (uint32_t)npx;
        WfConfig wc;
        std::memset(&wc, 0, sizeof wc);
        wc.tie = p->tie_mode;
        wc.bvh = s.bvh ? 1 : 0;
        wc.stats = 1;
        wc.block = wblock;
        uint32_t wstack = stack;
        r = pick_width(c, p, wstack, wc.wide);
        if (r != TRACER_OK) return r;
        a.stack_depth = wstack;
        if (wc.wide == WF_WIDTH_8) wc.cw8_stack = s.cw8_depth;
        if (wc.wide != WF_WIDTH_8) a.sc.tri_cw8 = a.sc.tri_cw8_prims = nullptr;
        const AdjWf aw{dldi, lin, ab.grad.p, s.nm, ab.pix.p, use_log ? ab.log.p : nullptr};
        c->last_kernel = TRACER_KERNEL_WAVEFRONT;
        c->last_launches = 1;  // + generate, rounds; the FP64-to-float conversion
        if (c->profiling) cudaEventRecord(c->prof_begin, st);
        // a sample takes at most max_depth rounds in each pass
        r = run_wavefront(c, a, wc, npx, 2 * (uint64_t)p->spp * p->max_depth + 1, wstack, p->wavefront, p->tail_paths, st, &aw);
        if (r != TRACER_OK) return r;
    } else {
        c->last_kernel = 3;
        c->last_launches = 2;  // adjoint + FP64-to-float conversion
        if (c->profiling) cudaEventRecord(c->prof_begin, st);
        e = launch_adjoint(a, dldi, lin, ab.grad.p, s.nm, p->tie_mode, s.bvh ? 1 : 0, st);
    }
    // the camera's boundary term: triangle outlines moving across pixels
    if (e == cudaSuccess && edges) {
        EdgeArgs ea{dldi, ab.grad.p + 6 * (size_t)s.nm, {}, c->edge_samples, 0.01f, ab.segs.p, ab.nsegs.p, seg_cap};
        if (!camera_inverse(f->camera, ea.binv)) return fail(c, TRACER_ERR_INVALID_ARG, "degenerate camera basis");
        TraceArgs ae = a;
        ae.stack_depth = stack;  // the binary traversal's
        e = launch_edge_campos(ae, ea, p->tie_mode, s.bvh ? 1 : 0, st);
        c->last_launches += 2;
    }
    if (c->profiling) cudaEventRecord(c->prof_end, st);
    if (e == cudaSuccess) e = launch_grad_to_float(ab.grad.p, ab.gradf.p, (uint32_t)ng, st);
    if (e == cudaSuccess) e = cudaEventRecord(c->done, st);
    if (e != cudaSuccess) return cuda_fail(c, e, "adjoint launch");
    c->pending = true;
    // outputs: device pointers get asynchronous copies, host pointers wait
    float* outs[3] = {d_albedo, d_emission, d_campos};
    const size_t offs[3] = {0, 3 * (size_t)s.nm, 6 * (size_t)s.nm};
    const size_t lens[3] = {3 * (size_t)s.nm, 3 * (size_t)s.nm, 3};
    bool host_out = false;
    for (int k = 0; k < 3; ++k) {
        if (!outs[k]) continue;
        if (is_device_ptr(outs[k])) {
            e = cudaMemcpyAsync(outs[k], ab.gradf.p + offs[k], lens[k] * sizeof(float), cudaMemcpyDeviceToDevice, st);
            if (e != cudaSuccess) return cuda_fail(c, e, "gradient copy");
        } else {
            host_out = true;
        }
    }
    if (e == cudaSuccess) e = cudaEventRecord(c->done, st);
    if (e != cudaSuccess) return cuda_fail(c, e, "adjoint completion event");
    if (host_out) {
        r = finish(c);
        if (r != TRACER_OK) return r;
        for (int k = 0; k < 3; ++k)
            if (outs[k] && !is_device_ptr(outs[k])) {
                e = cudaMemcpy(outs[k], ab.gradf.p + offs[k], lens[k] * sizeof(float), cudaMemcpyDeviceToHost);
                if (e != cudaSuccess) return cuda_fail(c, e, "gradient readback");
            }
    }
    return TRACER_OK;
}

// ------------------------------------------------------------------ present
namespace {

int check_present(tracer_ctx* c, const tracer_present_params* pp, size_t out_bytes)
{
    if (!pp) return fail(c, TRACER_ERR_INVALID_ARG, "null present params");
    if (pp->width == 0 || pp->height == 0 || pp->width > 32768 || pp->height > 32768)
        return fail(c, TRACER_ERR_NO_SUITABLE_SURFACE, "framebuffer %ux%u not supported", pp->width, pp->height);
    if (pp->out_aov != TRACER_AOV_RGBA8 && pp->out_aov != TRACER_AOV_RGBA32F)
        return fail(c, TRACER_ERR_NO_SUITABLE_SURFACE, "present output must be RGBA8 or RGBA32F");
    const size_t need = (size_t)pp->width * pp->height * (pp->out_aov == TRACER_AOV_RGBA8 ? 4 : 16);
    if (out_bytes < need) return fail(c, TRACER_ERR_INVALID_ARG, "output holds %zu bytes, needs %zu", out_bytes, need);
    return TRACER_OK;
}

// The present pass from device images into out (device: asynchronous; host:
// through the staging buffer, waiting for the result).
// With profiling on, tracer_last_timings' total_ms then covers the present
// kernel alone (own_timing) or the whole draw (the trace recorded the start).
int present_into(tracer_ctx* c, const tracer_present_params* pp, const void* img0, const void* img1, uint32_t sw,
                 uint32_t sh, int src_float, void* out, cudaStream_t st, bool own_timing)
{
    const size_t bytes = (size_t)pp->width * pp->height * (pp->out_aov == TRACER_AOV_RGBA8 ? 4 : 16);
    const bool dev_out = is_device_ptr(out);
    void* dst = out;
    cudaError_t e = cudaSuccess;
    if (!dev_out) {
        e = dalloc(c->pres_out, bytes);
        dst = c->pres_out.p;
    }
    if (e != cudaSuccess) return cuda_fail(c, e, "present staging allocation");
    PresentArgs pa{sw, sh, pp->width, pp->height,
                   pp->out_aov == TRACER_AOV_RGBA8 ? static_cast<uchar4*>(dst) : nullptr,
                   pp->out_aov == TRACER_AOV_RGBA32F ? static_cast<float4*>(dst) : nullptr};
    if (c->profiling && own_timing) cudaEventRecord(c->prof_begin, st);
    e = launch_present(pa, img0, img1, src_float, st);
    if (c->profiling) cudaEventRecord(c->prof_end, st);
    c->last_launches += 1;
    if (e == cudaSuccess) e = cudaEventRecord(c->done, st);
    if (e != cudaSuccess) return cuda_fail(c, e, "present launch");
    c->pending = true;
    if (!dev_out) {
        int r = finish(c);
        if (r != TRACER_OK) return r;
        e = cudaMemcpy(out, dst, bytes, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_fail(c, e, "present readback");
    }
    return TRACER_OK;
}

// Frame slots and accumulation buffers for w x h frames, cleared.
cudaError_t reset_draw(tracer_ctx* c, uint32_t w, uint32_t h, cudaStream_t st)
{
    const size_t npx = (size_t)w * h;
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < 2 && e == cudaSuccess; ++k) {
        e = dalloc(c->slot[k], npx);
        if (e == cudaSuccess) e = cudaMemsetAsync(c->slot[k].p, 0, npx * sizeof(uchar4), st);
    }
    c->slot_w = w;
    c->slot_h = h;
    c->draw_frame = 0;
    c->acc_n = 0;
    return e;
}

}  // namespace

extern "C" int tracer_present(tracer_ctx* c, const void* image0, const void* image1, uint32_t src_width,
                              uint32_t src_height, int src_aov, const tracer_present_params* pp, void* out,
                              size_t out_bytes, void* cuda_stream)
{
    if (!c) return TRACER_ERR_INVALID_ARG;
    if (!image0 || !image1 || !out) return fail(c, TRACER_ERR_INVALID_ARG, "null image or output");
    int r = check_present(c, pp, out_bytes);
    if (r != TRACER_OK) return r;
    if (src_aov != TRACER_AOV_RGBA8 && src_aov != TRACER_AOV_RGBA32F)
        return fail(c, TRACER_ERR_NO_SUITABLE_SURFACE, "source images must be RGBA8 or RGBA32F");
    if (src_width == 0 || src_height == 0 || src_width > 32768 || src_height > 32768)
        return fail(c, TRACER_ERR_NO_SUITABLE_SURFACE, "source %ux%u not supported", src_width, src_height);
    r = finish(c);  // the staging buffers may still be read by the last call
    if (r != TRACER_OK) return r;
    cudaSetDevice(c->device);
    cudaStream_t st = cuda_stream ? static_cast<cudaStream_t>(cuda_stream) : c->stream;
    const size_t sbytes = (size_t)src_width * src_height * (src_aov == TRACER_AOV_RGBA8 ? 4 : 16);
    const void* src[2] = {image0, image1};
    for (int k = 0; k < 2; ++k) {
        if (is_device_ptr(src[k])) continue;
        cudaError_t e = dalloc(c->pres_src[k], sbytes);
        if (e == cudaSuccess) e = cudaMemcpyAsync(c->pres_src[k].p, src[k], sbytes, cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) return cuda_fail(c, e, "present source upload");
        src[k] = c->pres_src[k].p;
    }
    c->last_launches = 0;
    c->last_kernel = 0;
    c->last_rounds = 0;
    c->last_prof_rounds = 0;
    c->last_round_entries = 0;
    c->last_finish = false;
    return present_into(c, pp, src[0], src[1], src_width, src_height, src_aov == TRACER_AOV_RGBA32F, out, st, true);
}

extern "C" int tracer_draw(tracer_ctx* c, const tracer_frame* f, const tracer_trace_params* p,
                           const tracer_present_params* pp, void* out, size_t out_bytes, void* cuda_stream)
{
    if (!c) return TRACER_ERR_INVALID_ARG;
    if (!f || !p || !out) return fail(c, TRACER_ERR_INVALID_ARG, "null frame, params or output");
    int r = check_present(c, pp, out_bytes);
    if (r != TRACER_OK) return r;
    if (pp->mode != TRACER_PRESENT_PINGPONG && pp->mode != TRACER_PRESENT_ACCUMULATE)
        return fail(c, TRACER_ERR_INVALID_ARG, "unknown present mode %u", pp->mode);
    const bool accumulate = pp->mode == TRACER_PRESENT_ACCUMULATE;
    tracer_trace_params q = *p;
    q.aov_mask = (q.aov_mask ? q.aov_mask : (1u << TRACER_AOV_RGBA8)) | (1u << TRACER_AOV_RGBA8) |
                 (accumulate ? 1u << TRACER_AOV_LINEAR : 0u);
    cudaStream_t st = cuda_stream ? static_cast<cudaStream_t>(cuda_stream) : c->stream;
    const size_t npx = (size_t)q.width * q.height;
    if (q.width != c->slot_w || q.height != c->slot_h || !c->slot[0].p) {
        r = finish(c);
        if (r != TRACER_OK) return r;
        cudaSetDevice(c->device);
        cudaError_t e = reset_draw(c, q.width, q.height, st);
        if (e != cudaSuccess) return cuda_fail(c, e, "frame slot allocation");
    }
    r = tracer_trace(c, f, &q, cuda_stream);
    if (r != TRACER_OK) return r;
    cudaError_t e = cudaSuccess;
    if (!accumulate) {
        // frame k's image goes to slot k % 2; the pass reads the slots as bound
        const int s = (int)(c->draw_frame & 1);
        e = cudaMemcpyAsync(c->slot[s].p, c->rgba8.p, npx * sizeof(uchar4), cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) return cuda_fail(c, e, "frame slot copy");
        r = present_into(c, pp, c->slot[0].p, c->slot[1].p, q.width, q.height, 0, out, st, false);
    } else {
        // the camera's four vectors, bit for bit (not its padding lanes)
        const tracer_camera &ca = c->acc_frame.camera, &cb = f->camera;
        const bool same_cam = std::memcmp(ca.pos, cb.pos, sizeof ca.pos) == 0 &&
                              std::memcmp(ca.dir, cb.dir, sizeof ca.dir) == 0 &&
                              std::memcmp(ca.right, cb.right, sizeof ca.right) == 0 &&
                              std::memcmp(ca.up, cb.up, sizeof ca.up) == 0;
        const bool same = c->acc_n > 0 && c->acc_version == c->scene_version &&
                          c->acc_frame.aspect_ratio == f->aspect_ratio && same_cam &&
                          c->acc_params.spp == q.spp && c->acc_params.max_depth == q.max_depth &&
                          c->acc_params.rr_start == q.rr_start && c->acc_params.tie_mode == q.tie_mode &&
                          std::memcmp(c->acc_params.sky, q.sky, sizeof q.sky) == 0;
        if (!same) {
            e = dalloc(c->acc_sum, npx);
            if (e == cudaSuccess) e = dalloc(c->acc_disp[0], npx);
            if (e == cudaSuccess) e = dalloc(c->acc_disp[1], npx);
            if (e == cudaSuccess) e = cudaMemsetAsync(c->acc_sum.p, 0, npx * sizeof(float4), st);
            if (e == cudaSuccess) e = cudaMemsetAsync(c->acc_disp[0].p, 0, npx * sizeof(float4), st);
            if (e == cudaSuccess) e = cudaMemsetAsync(c->acc_disp[1].p, 0, npx * sizeof(float4), st);
            if (e != cudaSuccess) return cuda_fail(c, e, "accumulation buffers");
            c->acc_n = 0;
            c->acc_frame = *f;
            c->acc_params = q;
            c->acc_version = c->scene_version;
        }
        ++c->acc_n;
        const int cur = (int)(c->acc_n & 1);
        e = launch_accumulate(c->linear.p, c->acc_sum.p, c->acc_disp[cur].p, (uint32_t)npx, c->acc_n, c->sm_count,
                              st);
        c->last_launches += 1;
        if (e != cudaSuccess) return cuda_fail(c, e, "accumulate launch");
        r = present_into(c, pp, c->acc_disp[cur].p, c->acc_disp[cur ^ 1].p, q.width, q.height, 1, out, st, false);
    }
    if (r == TRACER_OK) ++c->draw_frame;
    return r;
}

extern "C" int tracer_draw_reset(tracer_ctx* c)
{
    if (!c) return TRACER_ERR_INVALID_ARG;
    int r = finish(c);
    if (r != TRACER_OK) return r;
    cudaSetDevice(c->device);
    if (c->slot_w && c->slot_h) {
        cudaError_t e = reset_draw(c, c->slot_w, c->slot_h, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) return cuda_fail(c, e, "draw reset");
    }
    c->draw_frame = 0;
    c->acc_n = 0;
    return TRACER_OK;
}

// ------------------------------------------------------------ legacy Whitted
extern "C" int tracer_trace_whitted(tracer_ctx* c, const tracer_frame* f, const tracer_trace_params* p,
                                    void* cuda_stream)
{
    if (!c) return TRACER_ERR_INVALID_ARG;
    if (!f || !p) return fail(c, TRACER_ERR_INVALID_ARG, "null frame or params");
    if (p->width == 0 || p->height == 0 || p->width > 32768 || p->height > 32768)
        return fail(c, TRACER_ERR_NO_SUITABLE_SURFACE, "image size %ux%u not supported", p->width, p->height);
    const uint32_t mask = p->aov_mask ? p->aov_mask : (1u << TRACER_AOV_RGBA8);
    if (mask & ~((1u << TRACER_AOV_RGBA8) | (1u << TRACER_AOV_RGBA32F) | (1u << TRACER_AOV_STATS)))
        return fail(c, TRACER_ERR_NO_SUITABLE_SURFACE, "the Whitted shader writes RGBA8, RGBA32F and STATS only");
    int r = finish(c);
    if (r != TRACER_OK) return r;
    cudaSetDevice(c->device);
    const size_t npx = (size_t)p->width * p->height;
    cudaError_t e = cudaSuccess;
    if (mask & (1u << TRACER_AOV_RGBA8)) e = dalloc(c->rgba8, npx);
    if (e == cudaSuccess && (mask & (1u << TRACER_AOV_RGBA32F))) e = dalloc(c->rgba32f, npx);
    if (e != cudaSuccess) return cuda_fail(c, e, "image allocation");
    TraceArgs a;
    std::memset(&a, 0, sizeof a);
    a.fr.aspect = f->aspect_ratio;
    a.fr.seed = f->seed;
    a.fr.cpos = V3{f->camera.pos[0], f->camera.pos[1], f->camera.pos[2]};
    a.fr.cdir = V3{f->camera.dir[0], f->camera.dir[1], f->camera.dir[2]};
    a.fr.cright = V3{f->camera.right[0], f->camera.right[1], f->camera.right[2]};
    a.fr.cup = V3{f->camera.up[0], f->camera.up[1], f->camera.up[2]};
    a.fr.light = V3{f->light_pos[0], f->light_pos[1], f->light_pos[2]};
    a.width = p->width;
    a.height = p->height;
    a.rgba8 = (mask & (1u << TRACER_AOV_RGBA8)) ? c->rgba8.p : nullptr;
    a.rgba32f = (mask & (1u << TRACER_AOV_RGBA32F)) ? c->rgba32f.p : nullptr;
    a.stats = c->stats.p;
    a.status = c->status.p;
    const int stats = (p->stats || (mask & (1u << TRACER_AOV_STATS))) ? 1 : 0;
    cudaStream_t st = cuda_stream ? static_cast<cudaStream_t>(cuda_stream) : c->stream;
    e = cudaMemsetAsync(c->stats.p, 0, sizeof(unsigned long long) * C_COUNT, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->status.p, 0, sizeof(int), st);
    if (e != cudaSuccess) return cuda_fail(c, e, "trace set-up");
    c->width = p->width;
    c->height = p->height;
    c->last_mask = mask | (stats ? (1u << TRACER_AOV_STATS) : 0u);
    c->last_kernel = 0;
    c->last_rounds = 0;
    c->last_prof_rounds = 0;
    c->last_round_entries = 0;
    c->last_finish = false;
    c->last_launches = 1;
    if (c->profiling) cudaEventRecord(c->prof_begin, st);
    e = launch_whitted(a, stats, st);
    if (c->profiling) cudaEventRecord(c->prof_end, st);
    if (e == cudaSuccess) e = cudaEventRecord(c->done, st);
    if (e != cudaSuccess) return cuda_fail(c, e, "Whitted launch");
    c->pending = true;
    return TRACER_OK;
}
