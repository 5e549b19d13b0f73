// gkrt_api.cu — host side of the C ABI declared in include/gkrt.h.
//
// Mirrors the lifecycle of the reference's path-tracing logic renderer
// (src/Rendering/PathTracing/PathTracingRenderer.cpp:18-232): create, (re)size images,
// load a scene, build acceleration structures, then per frame: rt pass -> reproject pass
// -> compose pass -> history hand-over. Every entry point returns a status code; no
// exception crosses the boundary.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "gk_shade.cuh"
#include "gk_tma.cuh"
#include "gkrt_internal.h"

using namespace gk;

// Staging tables: 0 instance materials, 1 previous transforms, 2 DevInst, 3 emitter geometry,
// 4 emitter alias table, 5 refit transforms.
constexpr int kStageSlots = 6;
struct StageSlot {
    void* p[2] = {nullptr, nullptr};
    size_t cap[2] = {0, 0};
    cudaEvent_t ev[2] = {nullptr, nullptr};
    int cur = 0;
};

// Pass scopes, named as the reference's GPU timer scopes (PathTracingRenderer.cpp:111, 126, 138,
// 160; RayTraceBaseRenderer.cpp:209).
enum PassId { kPassRt, kPassReproject, kPassCompose, kPassCopy, kPassTlas, kPassCount };
static const char* const kPassNames[kPassCount] = {"rt pass", "reproject pass", "compose pass", "copy pass",
                                                   "TLAS Update"};

struct GkrtContext {
    int device = 0;
    bool timers = false;                        // GKRT_DEVICE_PASS_TIMERS
    cudaEvent_t pass_ev[kPassCount][2] = {};    // begin / end of each pass's last run
    bool pass_recorded[kPassCount] = {};
    uint32_t watchdog_ms = 60000;
    std::string err;
    uint32_t W = 0, H = 0, P = 0;     // P: row pitch in pixels (W rounded up to 4: 16-byte rows)
    void* img[GKRT_IMG_COUNT] = {};
    float4* atrous_tmp[2] = {nullptr, nullptr};   // ping-pong of the a-trous passes
    uint32_t* d_output = nullptr;     // presentation image, OW x OH BGRA8 words (gkrt_output_resize)
    uint32_t OW = 0, OH = 0;

    bool has_scene = false;
    std::vector<GkrtMesh> meshes;
    std::vector<GkrtInstance> inst;
    std::vector<float> pos_host;      // float4 per vertex (kept for BVH builds)
    std::vector<uint32_t> idx_host;
    std::vector<GkrtMaterial> mat_host;
    std::vector<std::vector<uint32_t>> slot_tris;   // per mesh and material slot
    float4* d_emit = nullptr;         // emissive-triangle table (GKRT_NEE_EMISSIVE)
    float2* d_emit_alias = nullptr;
    uint32_t nemit = 0, emit_cap = 0;
    uint32_t nvert = 0, nidx = 0, nmat = 0;
    float4* d_pos = nullptr;
    float4* d_nrm = nullptr;
    float2* d_uv = nullptr;           // texture coordinates (optional)
    float4* d_tan = nullptr;          // object-space tangents (optional)
    bool textured = false;            // some material names a texture
    uint32_t* d_slot = nullptr;
    uint32_t* d_idx = nullptr;
    GkrtMaterial* d_mat = nullptr;
    uint32_t* d_inst_mat = nullptr;
    float* d_inst_prev = nullptr;
    DevInst* d_inst = nullptr;
    uint32_t* d_cubes = nullptr;                // probe grid (uploaded, or made by gkrt_probe_voxelize)
    uint32_t* d_voxels = nullptr;
    uint32_t* d_cubes_prev = nullptr;           // snapshot the bake interpolates from
    // page-locked staging of the per-update tables (instance tables, emitter table, refit
    // transforms), so that their uploads are asynchronous on the caller's stream: two buffers
    // per table, each with the event recorded after its last upload
    StageSlot stage[kStageSlots];
    std::vector<GkrtLight> lights_host;

    // acceleration structures: d_nodes holds the builders' two-child mesh-level nodes
    // [0, blas_node_count) and the instance-level nodes after them; d_wide holds their
    // collapse into the 8-wide nodes the kernels traverse (mesh level [0, blas_wide_count),
    // then the instance level)
    bool host_build = false;          // GKRT_BUILD_ON_HOST
    GpuBvh* builder = nullptr;
    uint32_t blas_node_count = 0, blas_nodes_used = 0;
    uint32_t tri_count = 0;           // triangles in d_tris
    std::vector<int> blas_root;
    std::vector<float> blas_box;      // 6 per mesh
    float* d_blas_box = nullptr;
    BvhNode* d_nodes = nullptr;
    size_t d_nodes_cap = 0;
    float4* d_tris = nullptr;
    int tlas_root = -1;
    uint32_t tlas_nodes = 0;
    WideNode* d_wide = nullptr;
    size_t d_wide_cap = 0;
    std::vector<int> blas_wide_root;
    uint32_t blas_wide_count = 0, tlas_wide_count = 0;
    int blas_wide_depth = 0, tlas_wide_depth = 0, tlas_wide_root = -1;
    int blas_bin_depth = 0, tlas_bin_depth = 0;   // two-child levels (root = 0)
    bool blas_ready = false, tlas_ready = false;
    uint32_t inst_cap = 0;            // instance arrays allocated for this many instances
    // instance-level refit: links recorded by the last instance-level collapse, scratch, and
    // which instances that build put in the tree
    RefitLinks refit;
    float* d_refit_ubox = nullptr;
    uint32_t* d_refit_arrive = nullptr;
    GpuInstBox* d_refit_inst = nullptr;
    size_t refit_ncap = 0, refit_wcap = 0, refit_icap = 0;
    std::vector<uint8_t> tlas_members;
    uint32_t tlas_refits = 0;
    uint32_t tlas_rebuilds = 0;
    // the refit-or-rebuild policy (gkrt_scene_update_instances_auto): each trace pass copies its
    // counters into one of two page-locked records (by pass parity) with an event after it
    unsigned long long* h_trace_counters = nullptr;   // 2 x 7, the Counters slots of d_counters
    cudaEvent_t trace_ev[2] = {};
    uint64_t trace_seq = 0;        // trace passes recorded
    uint64_t trace_seq_read = 0;   // passes the policy has read (their sequence numbers + 1)
    uint64_t base_after = 0;       // the baseline comes from a pass with this sequence number or later
    double visits_base = -1.0, visits_last = -1.0;   // node visits per ray; -1: none yet

    // the texture pool: one RGBA-float buffer per uploaded id and the device table the kernels
    // read (GKRT_MAX_TEXTURES entries, null texels for an id without a texture)
    std::vector<float4*> tex_buf;
    DevTex* d_tex = nullptr;
    // per texture id the nine-term spherical-harmonic projection of an RGBA32F texture (27
    // floats, see project_sky_sh), zero for 8-bit textures; empty until the first HDR upload
    std::vector<float> tex_sh;

    Unet* unet = nullptr;                       // learned denoiser (gkrt_unet_init)
    unsigned long long* d_counters = nullptr;   // see Counters (gk_trace.cuh): 6 per-pass slots + total rays
    uint32_t* d_error = nullptr;
    unsigned int* d_work = nullptr;             // pixel counter of the persistent trace kernel
    int num_sms = 1;
};

// Scope of one pass on its stream: an NVTX range, and with pass timers the begin and end events.
struct PassScope {
    GkrtContext* ctx;
    int id;
    cudaStream_t st;
    PassScope(GkrtContext* c, int i, cudaStream_t s) : ctx(c), id(i), st(s) {
        nvtxRangePushA(kPassNames[i]);
        if (ctx->timers) cudaEventRecord(ctx->pass_ev[i][0], st);
    }
    ~PassScope() {
        if (ctx->timers) {
            cudaEventRecord(ctx->pass_ev[id][1], st);
            ctx->pass_recorded[id] = true;
        }
        nvtxRangePop();
    }
};

namespace {

int fail(GkrtContext* c, int code, const std::string& msg) {
    if (c) c->err = msg;
    return code;
}

int cuda_fail(GkrtContext* c, cudaError_t e, const char* what) {
    int code = (e == cudaErrorMemoryAllocation) ? GKRT_ERR_OOM : GKRT_ERR_CUDA;
    return fail(c, code, std::string(what) + ": " + cudaGetErrorString(e));
}

#define GK_CUDA(call)                                             \
    do {                                                          \
        cudaError_t e_ = (call);                                  \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
    } while (0)

template <class T>
void dfree(T*& p) {
    if (p) cudaFree(p);
    p = nullptr;
}

size_t image_bytes_per_px(int id) {
    switch (id) {
        case GKRT_IMG_OBJECT_ID: case GKRT_IMG_OBJECT_ID_PREV: case GKRT_IMG_MOTION_MOMENT:
        case GKRT_IMG_HIT_INST: case GKRT_IMG_HIT_PRIM: case GKRT_IMG_PREV_DEPTH:
            return 4;
        case GKRT_IMG_MOTION:
            return 8;
        default:
            return 16;
    }
}
uint32_t image_format(int id) {
    switch (id) {
        case GKRT_IMG_OBJECT_ID: case GKRT_IMG_OBJECT_ID_PREV: case GKRT_IMG_MOTION_MOMENT:
        case GKRT_IMG_HIT_INST: case GKRT_IMG_HIT_PRIM:
            return GKRT_FMT_U32;
        case GKRT_IMG_PREV_DEPTH:
            return GKRT_FMT_F32;
        case GKRT_IMG_MOTION:
            return GKRT_FMT_F32X2;
        default:
            return GKRT_FMT_F32X4;
    }
}

void free_images(GkrtContext* c) {
    for (auto& p : c->img) dfree(p);
    dfree(c->atrous_tmp[0]);
    dfree(c->atrous_tmp[1]);
    c->W = c->H = c->P = 0;
}

void free_scene(GkrtContext* c) {
    dfree(c->d_pos); dfree(c->d_nrm); dfree(c->d_slot); dfree(c->d_idx); dfree(c->d_mat);
    dfree(c->d_uv); dfree(c->d_tan);
    c->textured = false;
    dfree(c->d_inst_mat); dfree(c->d_inst_prev); dfree(c->d_inst); dfree(c->d_cubes); dfree(c->d_voxels);
    dfree(c->d_cubes_prev);
    c->lights_host.clear();
    dfree(c->d_nodes); dfree(c->d_wide); dfree(c->d_tris); dfree(c->d_blas_box); dfree(c->d_emit); dfree(c->d_emit_alias);
    c->nemit = c->emit_cap = 0;
    c->mat_host.clear(); c->slot_tris.clear();
    c->d_nodes_cap = 0;
    c->d_wide_cap = 0;
    c->blas_wide_root.clear();
    c->blas_wide_count = c->tlas_wide_count = 0;
    c->blas_wide_depth = c->tlas_wide_depth = 0;
    c->blas_bin_depth = c->tlas_bin_depth = 0;
    c->tlas_wide_root = -1;
    c->inst_cap = 0;
    c->has_scene = false;
    c->blas_ready = c->tlas_ready = false;
    c->tlas_root = -1;
    c->blas_node_count = c->blas_nodes_used = 0;
    c->tri_count = 0;
    c->meshes.clear(); c->inst.clear(); c->pos_host.clear(); c->idx_host.clear();
    c->blas_root.clear(); c->blas_box.clear();
    dfree(c->refit.parent); dfree(c->refit.leaf); dfree(c->refit.wsrc);
    dfree(c->d_refit_ubox); dfree(c->d_refit_arrive); dfree(c->d_refit_inst);
    c->refit = RefitLinks();
    c->refit_ncap = c->refit_wcap = c->refit_icap = 0;
    c->tlas_members.clear();
}

template <class T>
int upload(GkrtContext* ctx, T*& dst, const void* src, size_t bytes) {
    dfree(dst);
    if (bytes == 0) return GKRT_OK;
    GK_CUDA(cudaMalloc((void**)&dst, bytes));
    GK_CUDA(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice));
    return GKRT_OK;
}

bool finite3(const float* p) { return std::isfinite(p[0]) && std::isfinite(p[1]) && std::isfinite(p[2]); }

int validate_instances(GkrtContext* ctx, const GkrtInstance* in, uint32_t n, uint32_t nmesh, uint32_t nmat) {
    for (uint32_t i = 0; i < n; ++i) {
        if (in[i].mesh_id >= nmesh) return fail(ctx, GKRT_ERR_INVALID_ARG, "instance mesh_id out of range");
        for (int k = 0; k < 16; ++k)
            if (in[i].mat_id[k] >= nmat && nmat > 0)
                return fail(ctx, GKRT_ERR_INVALID_ARG, "instance mat_id out of range");
        for (int k = 0; k < 12; ++k)
            if (!std::isfinite(in[i].world[k]) || !std::isfinite(in[i].world_inv[k]) ||
                !std::isfinite(in[i].combined_prev[k]))
                return fail(ctx, GKRT_ERR_INVALID_ARG, "non-finite instance transform");
        // world * world_inv must be the identity
        for (int r = 0; r < 3; ++r)
            for (int cc = 0; cc < 4; ++cc) {
                double s = (cc == 3) ? (double)in[i].world[4 * r + 3] : 0.0;
                for (int k = 0; k < 3; ++k) s += (double)in[i].world[4 * r + k] * (double)in[i].world_inv[4 * k + cc];
                double want = (r == cc) ? 1.0 : 0.0;
                double scale = 1.0 + std::fabs((double)in[i].world[4 * r + 3]);
                if (std::fabs(s - want) > 1e-3 * scale)
                    return fail(ctx, GKRT_ERR_INVALID_ARG, "world_inv is not the inverse of world");
            }
    }
    return GKRT_OK;
}

template <class T>
int copy_in(GkrtContext* ctx, T* dst, const void* src, size_t bytes) {
    if (bytes) GK_CUDA(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice));
    return GKRT_OK;
}

// Page-locked staging buffer of table `slot`, at least `bytes`: the other of its two buffers
// than the last call's, so the host waits only for the upload staged two updates ago.
void* stage_buf(GkrtContext* ctx, int slot, size_t bytes) {
    StageSlot& S = ctx->stage[slot];
    S.cur ^= 1;
    const int c = S.cur;
    if (S.ev[c]) cudaEventSynchronize(S.ev[c]);
    if (bytes > S.cap[c]) {
        if (S.p[c]) cudaFreeHost(S.p[c]);
        S.p[c] = nullptr;
        S.cap[c] = 0;
        const size_t cap = bytes + bytes / 4 + 256;
        if (cudaMallocHost(&S.p[c], cap) != cudaSuccess) {
            S.p[c] = nullptr;
            return nullptr;
        }
        S.cap[c] = cap;
    }
    return S.p[c];
}

// Upload of the buffer stage_buf(slot) returned last to dst, asynchronous on st; the slot's
// event is recorded after it.
int copy_staged(GkrtContext* ctx, int slot, void* dst, size_t bytes, cudaStream_t st) {
    StageSlot& S = ctx->stage[slot];
    if (bytes) GK_CUDA(cudaMemcpyAsync(dst, S.p[S.cur], bytes, cudaMemcpyHostToDevice, st));
    if (!S.ev[S.cur]) GK_CUDA(cudaEventCreateWithFlags(&S.ev[S.cur], cudaEventDisableTiming));
    GK_CUDA(cudaEventRecord(S.ev[S.cur], st));
    return GKRT_OK;
}

// Instance tables of the kernels; allocated once per scene (updates keep the count). Updates
// are built in page-locked memory and uploaded asynchronously on `st`.
int upload_instances(GkrtContext* ctx, cudaStream_t st) {
    const uint32_t n = (uint32_t)ctx->inst.size();
    uint32_t* mats = static_cast<uint32_t*>(stage_buf(ctx, 0, 64 * (size_t)n + 4));
    float* prev = static_cast<float*>(stage_buf(ctx, 1, 96 * (size_t)n + 4));
    DevInst* di = static_cast<DevInst*>(stage_buf(ctx, 2, sizeof(DevInst) * (size_t)n + 16));
    if (!mats || !prev || !di) return fail(ctx, GKRT_ERR_OOM, "page-locked staging of the instance tables");
    for (uint32_t i = 0; i < n; ++i) {
        const GkrtInstance& s = ctx->inst[i];
        std::memcpy(&mats[16 * (size_t)i], s.mat_id, 64);
        std::memcpy(&prev[24 * (size_t)i], s.combined_prev, 48);
        std::memcpy(&prev[24 * (size_t)i + 12], s.world, 48);
        std::memcpy(di[i].winv, s.world_inv, 48);
        const GkrtMesh& m = ctx->meshes[s.mesh_id];
        di[i].blas_root = ctx->blas_ready ? ctx->blas_root[s.mesh_id] : -1;
        di[i].blas_wide_root = ctx->blas_ready ? ctx->blas_wide_root[s.mesh_id] : -1;
        di[i].pad[0] = di[i].pad[1] = di[i].pad[2] = 0u;
        di[i].index_offset = m.index_offset;
        di[i].vertex_offset = m.vertex_offset;
        di[i].instance_id = s.instance_id;
    }
    int rc;
    if (ctx->inst_cap < n || !ctx->d_inst) {
        if ((rc = upload(ctx, ctx->d_inst_mat, mats, 64 * (size_t)n)) != GKRT_OK) return rc;
        if ((rc = upload(ctx, ctx->d_inst_prev, prev, 96 * (size_t)n)) != GKRT_OK) return rc;
        if ((rc = upload(ctx, ctx->d_inst, di, sizeof(DevInst) * (size_t)n)) != GKRT_OK) return rc;
        ctx->inst_cap = n;
        return GKRT_OK;
    }
    if ((rc = copy_staged(ctx, 0, ctx->d_inst_mat, 64 * (size_t)n, st)) != GKRT_OK) return rc;
    if ((rc = copy_staged(ctx, 1, ctx->d_inst_prev, 96 * (size_t)n, st)) != GKRT_OK) return rc;
    return copy_staged(ctx, 2, ctx->d_inst, sizeof(DevInst) * (size_t)n, st);
}

// d_nodes capacity for `total` nodes, keeping the mesh-level part.
int ensure_node_cap(GkrtContext* ctx, size_t total) {
    if (total <= ctx->d_nodes_cap && ctx->d_nodes) return GKRT_OK;
    const size_t cap = std::max<size_t>(total + total / 4, 16);
    BvhNode* q = nullptr;
    GK_CUDA(cudaMalloc((void**)&q, cap * sizeof(BvhNode)));
    cudaError_t e = cudaSuccess;
    if (ctx->d_nodes && ctx->blas_node_count)
        e = cudaMemcpy(q, ctx->d_nodes, (size_t)ctx->blas_node_count * sizeof(BvhNode), cudaMemcpyDeviceToDevice);
    if (e != cudaSuccess) {
        cudaFree(q);
        return cuda_fail(ctx, e, "cudaMemcpy(nodes)");
    }
    dfree(ctx->d_nodes);
    ctx->d_nodes = q;
    ctx->d_nodes_cap = cap;
    return GKRT_OK;
}

int get_builder(GkrtContext* ctx) {
    if (!ctx->builder) ctx->builder = gpu_bvh_new();
    return ctx->builder ? GKRT_OK : fail(ctx, GKRT_ERR_OOM, "BVH builder");
}

// d_wide capacity for `total` wide nodes, keeping the first `keep`.
int ensure_wide_cap(GkrtContext* ctx, size_t total, size_t keep) {
    if (total <= ctx->d_wide_cap && ctx->d_wide) return GKRT_OK;
    const size_t cap = std::max<size_t>(total + total / 4, 16);
    WideNode* q = nullptr;
    GK_CUDA(cudaMalloc((void**)&q, cap * sizeof(WideNode)));
    cudaError_t e = cudaSuccess;
    if (ctx->d_wide && keep) e = cudaMemcpy(q, ctx->d_wide, keep * sizeof(WideNode), cudaMemcpyDeviceToDevice);
    if (e != cudaSuccess) {
        cudaFree(q);
        return cuda_fail(ctx, e, "cudaMemcpy(wide nodes)");
    }
    dfree(ctx->d_wide);
    ctx->d_wide = q;
    ctx->d_wide_cap = cap;
    return GKRT_OK;
}

// Stack a ray can need: two-child traversal pushes at most one ref per level of each tree
// plus the marker; wide traversal one group per wide level plus the marker.
int check_stack_bound(GkrtContext* ctx) {
    if (ctx->blas_bin_depth + ctx->tlas_bin_depth + 3 > kStackSize)
        return fail(ctx, GKRT_ERR_DEVICE_LIMIT, "BVH deeper than the traversal stack allows (" +
                                                    std::to_string(ctx->blas_bin_depth) + " mesh + " +
                                                    std::to_string(ctx->tlas_bin_depth) + " instance levels)");
    if (ctx->blas_wide_depth + ctx->tlas_wide_depth + 1 > kStackEntries)
        return fail(ctx, GKRT_ERR_DEVICE_LIMIT, "BVH deeper than the traversal stack allows (" +
                                                    std::to_string(ctx->blas_wide_depth) + " mesh + " +
                                                    std::to_string(ctx->tlas_wide_depth) + " instance levels)");
    return GKRT_OK;
}

// The mesh-level two-child trees in d_nodes collapsed into wide nodes [0, blas_wide_count).
int finish_blas(GkrtContext* ctx, cudaStream_t st) {
    int rc = upload(ctx, ctx->d_blas_box, ctx->blas_box.data(), ctx->blas_box.size() * 4);
    if (rc != GKRT_OK) return rc;
    if ((rc = get_builder(ctx)) != GKRT_OK) return rc;
    const size_t cap = (size_t)ctx->blas_node_count + 2 * ctx->inst.size() + 2;
    dfree(ctx->d_wide);
    ctx->d_wide_cap = 0;
    if ((rc = ensure_wide_cap(ctx, cap, 0)) != GKRT_OK) return rc;
    const cudaError_t e = gpu_bvh_collapse(ctx->builder, ctx->d_nodes, ctx->blas_root, 0, ctx->d_wide, ctx->d_wide_cap,
                                           ctx->blas_wide_root, &ctx->blas_wide_count, &ctx->blas_wide_depth, st);
    if (e == cudaErrorInvalidValue)
        return fail(ctx, GKRT_ERR_INVALID_ARG, "mesh BVH collapse failed (non-finite geometry or depth > 64)");
    if (e != cudaSuccess) return cuda_fail(ctx, e, "gpu_bvh_collapse(mesh level)");
    ctx->tlas_wide_depth = 0;
    ctx->tlas_bin_depth = 0;
    if ((rc = check_stack_bound(ctx)) != GKRT_OK) return rc;
    ctx->blas_ready = true;
    ctx->tlas_ready = false;
    return GKRT_OK;
}

// Refit links and scratch for an instance level of `bin_count` two-child node slots, reset
// (parents and leaves -1, counters 0) on st before the collapse records the links.
int prepare_refit(GkrtContext* ctx, uint32_t bin_count, cudaStream_t st) {
    const size_t nc = std::max<size_t>(bin_count, 1), wc = nc + 1, ic = std::max<size_t>(ctx->inst.size(), 1);
    if (nc > ctx->refit_ncap) {
        dfree(ctx->refit.parent); dfree(ctx->d_refit_ubox); dfree(ctx->d_refit_arrive);
        ctx->refit_ncap = 0;
        GK_CUDA(cudaMalloc((void**)&ctx->refit.parent, nc * sizeof(int)));
        GK_CUDA(cudaMalloc((void**)&ctx->d_refit_ubox, nc * 12 * sizeof(float)));
        GK_CUDA(cudaMalloc((void**)&ctx->d_refit_arrive, nc * sizeof(uint32_t)));
        ctx->refit_ncap = nc;
    }
    if (wc > ctx->refit_wcap) {
        dfree(ctx->refit.wsrc);
        ctx->refit_wcap = 0;
        GK_CUDA(cudaMalloc((void**)&ctx->refit.wsrc, wc * 8 * sizeof(int)));
        ctx->refit_wcap = wc;
    }
    if (ic > ctx->refit_icap) {
        dfree(ctx->refit.leaf); dfree(ctx->d_refit_inst);
        ctx->refit_icap = 0;
        GK_CUDA(cudaMalloc((void**)&ctx->refit.leaf, ic * sizeof(int)));
        GK_CUDA(cudaMalloc((void**)&ctx->d_refit_inst, ic * sizeof(GpuInstBox)));
        ctx->refit_icap = ic;
    }
    GK_CUDA(cudaMemsetAsync(ctx->refit.parent, 0xFF, nc * sizeof(int), st));
    GK_CUDA(cudaMemsetAsync(ctx->d_refit_arrive, 0, nc * sizeof(uint32_t), st));
    GK_CUDA(cudaMemsetAsync(ctx->refit.leaf, 0xFF, ic * sizeof(int), st));
    ctx->refit.nbase = ctx->blas_node_count;
    ctx->refit.ncap = (uint32_t)nc;
    ctx->refit.ninst = (uint32_t)ctx->inst.size();
    ctx->refit.wbase = ctx->blas_wide_count;
    ctx->refit.wcap = (uint32_t)wc;
    return GKRT_OK;
}

// Per instance: whether the instance-level build puts it in the tree.
void tlas_members(const GkrtContext* ctx, std::vector<uint8_t>& m) {
    m.resize(ctx->inst.size());
    for (size_t i = 0; i < ctx->inst.size(); ++i)
        m[i] = (ctx->inst[i].visible && ctx->blas_root[ctx->inst[i].mesh_id] >= 0) ? 1 : 0;
}

// The instance-level two-child tree (root ctx->tlas_root) collapsed after the mesh level.
int finish_tlas(GkrtContext* ctx, uint32_t bin_count, cudaStream_t st) {
    int rc;
    if ((rc = get_builder(ctx)) != GKRT_OK) return rc;
    if ((rc = ensure_wide_cap(ctx, (size_t)ctx->blas_wide_count + bin_count + 1, ctx->blas_wide_count)) != GKRT_OK)
        return rc;
    if ((rc = prepare_refit(ctx, bin_count, st)) != GKRT_OK) return rc;
    tlas_members(ctx, ctx->tlas_members);
    std::vector<int> wr;
    const cudaError_t e = gpu_bvh_collapse(ctx->builder, ctx->d_nodes, std::vector<int>(1, ctx->tlas_root),
                                           ctx->blas_wide_count, ctx->d_wide, ctx->d_wide_cap, wr,
                                           &ctx->tlas_wide_count, &ctx->tlas_wide_depth, st, &ctx->refit);
    if (e == cudaErrorInvalidValue)
        return fail(ctx, GKRT_ERR_INVALID_ARG, "instance BVH collapse failed (non-finite transforms or depth > 64)");
    if (e != cudaSuccess) return cuda_fail(ctx, e, "gpu_bvh_collapse(instance level)");
    ctx->tlas_wide_root = wr[0];
    return check_stack_bound(ctx);
}

// Mesh-level trees on the GPU: one build over every mesh's triangles.
int build_blas_gpu(GkrtContext* ctx, cudaStream_t st) {
    const uint32_t nm = (uint32_t)ctx->meshes.size();
    ctx->blas_root.assign(nm, -1);
    ctx->blas_box.assign(6 * (size_t)nm, 0.0f);
    size_t ntri = 0;
    for (const GkrtMesh& m : ctx->meshes) ntri += m.index_count / 3;
    dfree(ctx->d_tris);
    if (ntri) GK_CUDA(cudaMalloc((void**)&ctx->d_tris, 3 * ntri * sizeof(float4)));
    ctx->tri_count = (uint32_t)ntri;
    int rc;
    if ((rc = get_builder(ctx)) != GKRT_OK) return rc;
    GpuBvhResult r;
    GK_CUDA(gpu_bvh_build_meshes(ctx->builder, ctx->d_pos, ctx->d_idx, ctx->meshes.data(), nm, 0, ctx->d_tris, &r, st));
    ctx->blas_root = r.root_node;
    ctx->blas_bin_depth = r.depth;
    if (nm) GK_CUDA(cudaMemcpy(ctx->blas_box.data(), r.root_box, 6 * (size_t)nm * 4, cudaMemcpyDeviceToHost));
    ctx->blas_node_count = r.node_count;
    ctx->blas_nodes_used = r.nodes_used;
    dfree(ctx->d_nodes);
    ctx->d_nodes_cap = 0;
    if ((rc = ensure_node_cap(ctx, (size_t)r.node_count + 2 * ctx->inst.size() + 2)) != GKRT_OK) return rc;
    if (r.node_count)
        GK_CUDA(cudaMemcpy(ctx->d_nodes, r.nodes, (size_t)r.node_count * sizeof(BvhNode), cudaMemcpyDeviceToDevice));
    return finish_blas(ctx, st);
}

// Mesh-level trees on the host (GKRT_BUILD_ON_HOST).
int build_blas_host(GkrtContext* ctx, cudaStream_t st) {
    const uint32_t nm = (uint32_t)ctx->meshes.size();
    ctx->blas_bin_depth = 0;
    std::vector<BvhNode> nodes;
    ctx->blas_root.assign(nm, -1);
    ctx->blas_box.assign(6 * (size_t)nm, 0.0f);
    std::vector<float4> tris;
    for (uint32_t mi = 0; mi < nm; ++mi) {
        const GkrtMesh& m = ctx->meshes[mi];
        const uint32_t nt = m.index_count / 3;
        std::vector<float> boxes(6 * (size_t)nt);
        float rb[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
        for (uint32_t t = 0; t < nt; ++t) {
            for (int k = 0; k < 3; ++k) { boxes[6 * t + k] = INFINITY; boxes[6 * t + 3 + k] = -INFINITY; }
            for (int v = 0; v < 3; ++v) {
                const float* p = &ctx->pos_host[4 * (size_t)(ctx->idx_host[m.index_offset + 3 * t + v] + m.vertex_offset)];
                for (int k = 0; k < 3; ++k) {
                    boxes[6 * t + k] = std::min(boxes[6 * t + k], p[k]);
                    boxes[6 * t + 3 + k] = std::max(boxes[6 * t + 3 + k], p[k]);
                }
            }
            for (int k = 0; k < 3; ++k) {
                rb[k] = std::min(rb[k], boxes[6 * t + k]);
                rb[3 + k] = std::max(rb[3 + k], boxes[6 * t + 3 + k]);
            }
        }
        std::memcpy(&ctx->blas_box[6 * (size_t)mi], rb, sizeof(rb));
        if (nt == 0) continue;
        HostBvh hb;
        build_bvh_host(boxes.data(), nt, 4, (uint32_t)nodes.size(), (uint32_t)(tris.size() / 3), false, hb);
        ctx->blas_root[mi] = hb.root;
        ctx->blas_bin_depth = std::max(ctx->blas_bin_depth, hb.depth);
        nodes.insert(nodes.end(), hb.nodes.begin(), hb.nodes.end());
        for (uint32_t k = 0; k < nt; ++k) {
            const uint32_t prim = hb.order[k];
            for (int v = 0; v < 3; ++v) {
                const float* p = &ctx->pos_host[4 * (size_t)(ctx->idx_host[m.index_offset + 3 * prim + v] + m.vertex_offset)];
                float w = 0.0f;
                if (v == 0) std::memcpy(&w, &prim, 4);
                tris.push_back(make_float4(p[0], p[1], p[2], w));
            }
        }
    }
    int rc = upload(ctx, ctx->d_tris, tris.data(), tris.size() * sizeof(float4));
    if (rc != GKRT_OK) return rc;
    ctx->tri_count = (uint32_t)(tris.size() / 3);
    ctx->blas_node_count = ctx->blas_nodes_used = (uint32_t)nodes.size();
    dfree(ctx->d_nodes);
    ctx->d_nodes_cap = 0;
    if ((rc = ensure_node_cap(ctx, nodes.size() + 2 * ctx->inst.size() + 2)) != GKRT_OK) return rc;
    if ((rc = copy_in(ctx, ctx->d_nodes, nodes.data(), nodes.size() * sizeof(BvhNode))) != GKRT_OK) return rc;
    return finish_blas(ctx, st);
}

int build_blas(GkrtContext* ctx, cudaStream_t st) {
    return ctx->host_build ? build_blas_host(ctx, st) : build_blas_gpu(ctx, st);
}

// during (optional): host work run while the GPU builds the level (else before the build).
int build_tlas(GkrtContext* ctx, cudaStream_t st, int (*during)(GkrtContext*, cudaStream_t) = nullptr) {
    const uint32_t n = (uint32_t)ctx->inst.size();
    const uint32_t base = ctx->blas_node_count;
    int rc;
    const bool coop = !ctx->host_build && gpu_bvh_cooperative_supported();
    if (during && !coop && (rc = during(ctx, st)) != GKRT_OK) return rc;   // the host builder
    if (!ctx->host_build) {
        if ((rc = get_builder(ctx)) != GKRT_OK) return rc;
        // the instance tables first: their host work and uploads overlap the stream's earlier work
        if ((rc = upload_instances(ctx, st)) != GKRT_OK) return rc;
        if (coop) {
            // the tree's members, staged in page-locked memory and uploaded into the refit's
            // instance buffer (a refit rewrites it whole); one cooperative launch builds and
            // collapses the level; the host waits once
            uint32_t m = 0;
            for (uint32_t i = 0; i < n; ++i) m += (ctx->inst[i].visible && ctx->blas_root[ctx->inst[i].mesh_id] >= 0);
            const uint32_t slots = m + 1u;
            if ((rc = ensure_node_cap(ctx, (size_t)base + slots)) != GKRT_OK) return rc;
            if ((rc = ensure_wide_cap(ctx, (size_t)ctx->blas_wide_count + slots + 1, ctx->blas_wide_count)) != GKRT_OK)
                return rc;
            if ((rc = prepare_refit(ctx, slots, st)) != GKRT_OK) return rc;
            tlas_members(ctx, ctx->tlas_members);
            GpuInstBox* hb = static_cast<GpuInstBox*>(stage_buf(ctx, 5, sizeof(GpuInstBox) * (size_t)m + 16));
            if (!hb) return fail(ctx, GKRT_ERR_OOM, "page-locked staging of the instance boxes");
            uint32_t k = 0;
            for (uint32_t i = 0; i < n; ++i) {
                const GkrtInstance& in = ctx->inst[i];
                if (!in.visible || ctx->blas_root[in.mesh_id] < 0) continue;
                std::memcpy(hb[k].world, in.world, 48);
                hb[k].mesh = in.mesh_id;
                hb[k].inst = i;
                hb[k].pad0 = hb[k].pad1 = 0;
                ++k;
            }
            if ((rc = copy_staged(ctx, 5, ctx->d_refit_inst, sizeof(GpuInstBox) * (size_t)m, st)) != GKRT_OK) return rc;
            GK_CUDA(gpu_bvh_build_instance_level_launch(ctx->builder, ctx->d_refit_inst, m, ctx->d_blas_box, ctx->d_nodes,
                                                        base, slots, ctx->d_wide, ctx->blas_wide_count,
                                                        (uint32_t)ctx->d_wide_cap, &ctx->refit, st));
            // host work of the caller's (the emitter table) while the build runs
            const int rc_during = during ? during(ctx, st) : GKRT_OK;
            InstLevelResult r;
            GK_CUDA(gpu_bvh_build_instance_level_finish(ctx->builder, &r, st));
            if (r.error)
                return fail(ctx, GKRT_ERR_INVALID_ARG,
                            "instance BVH build failed (non-finite transforms or depth > 64), code " +
                                std::to_string(r.error));
            ctx->tlas_root = m ? (int)base : -1;
            ctx->tlas_nodes = r.nodes_used;
            ctx->tlas_bin_depth = r.depth;
            ctx->tlas_wide_root = m ? (int)ctx->blas_wide_count : -1;
            ctx->tlas_wide_count = r.wide_count;
            ctx->tlas_wide_depth = r.wide_depth;
            if ((rc = check_stack_bound(ctx)) != GKRT_OK) return rc;
            ctx->tlas_ready = true;
            ++ctx->tlas_rebuilds;
            return rc_during;
        }
        return fail(ctx, GKRT_ERR_NO_DEVICE, "the GPU instance-level build needs cooperative launches");
    }
    std::vector<float> boxes;
    std::vector<uint32_t> map;
    for (uint32_t i = 0; i < n; ++i) {
        const GkrtInstance& in = ctx->inst[i];
        if (!in.visible || ctx->blas_root[in.mesh_id] < 0) continue;
        const float* rb = &ctx->blas_box[6 * (size_t)in.mesh_id];
        double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int c = 0; c < 8; ++c) {
            double p[3] = {(c & 1) ? rb[3] : rb[0], (c & 2) ? rb[4] : rb[1], (c & 4) ? rb[5] : rb[2]};
            for (int r = 0; r < 3; ++r) {
                double v = (double)in.world[4 * r] * p[0] + (double)in.world[4 * r + 1] * p[1] +
                           (double)in.world[4 * r + 2] * p[2] + (double)in.world[4 * r + 3];
                lo[r] = std::min(lo[r], v);
                hi[r] = std::max(hi[r], v);
            }
        }
        // widen: the mesh level traverses the FP32-transformed ray, whose points sit within
        // rounding of the world ray's
        for (int r = 0; r < 3; ++r) {
            double pad = 1e-5 * (std::fabs(lo[r]) + std::fabs(hi[r]) + (hi[r] - lo[r])) + 1e-7;
            boxes.push_back((float)(lo[r] - pad));
        }
        for (int r = 0; r < 3; ++r) {
            double pad = 1e-5 * (std::fabs(lo[r]) + std::fabs(hi[r]) + (hi[r] - lo[r])) + 1e-7;
            boxes.push_back((float)(hi[r] + pad));
        }
        map.push_back(i);
    }
    HostBvh hb;
    build_bvh_host(boxes.data(), (uint32_t)map.size(), 1, base, 0, true, hb);
    // leaf payloads hold positions in `map`; rewrite them to instance indices
    for (auto& nd : hb.nodes) {
        int* r[2] = {&nd.d.x, &nd.d.y};
        for (int k = 0; k < 2; ++k)
            if (*r[k] < 0 && *r[k] != kRefPop) {
                uint32_t payload = ~(uint32_t)(*r[k]);
                uint32_t pos = payload >> 3;
                *r[k] = (int)(~(map[pos] << 3));
            }
    }
    if ((rc = ensure_node_cap(ctx, (size_t)base + hb.nodes.size())) != GKRT_OK) return rc;
    if ((rc = copy_in(ctx, ctx->d_nodes + base, hb.nodes.data(), hb.nodes.size() * sizeof(BvhNode))) != GKRT_OK)
        return rc;
    ctx->tlas_root = map.empty() ? -1 : hb.root;
    ctx->tlas_nodes = (uint32_t)hb.nodes.size();
    ctx->tlas_bin_depth = hb.depth;
    if ((rc = finish_tlas(ctx, (uint32_t)hb.nodes.size(), st)) != GKRT_OK) return rc;
    ctx->tlas_ready = true;
    ++ctx->tlas_rebuilds;
    return upload_instances(ctx, st);
}

// Instance-level refit in place, for instances that keep the members of the last build: the
// instance tables and the transforms staged and uploaded, then the two refit launches, all
// asynchronous on st (no host synchronisation).
int refit_tlas(GkrtContext* ctx, cudaStream_t st) {
    const uint32_t n = (uint32_t)ctx->inst.size();
    int rc;
    if ((rc = upload_instances(ctx, st)) != GKRT_OK) return rc;
    GpuInstBox* hb = static_cast<GpuInstBox*>(stage_buf(ctx, 5, sizeof(GpuInstBox) * (size_t)n + 16));
    if (!hb) return fail(ctx, GKRT_ERR_OOM, "page-locked staging of the refit transforms");
    for (uint32_t i = 0; i < n; ++i) {
        std::memcpy(hb[i].world, ctx->inst[i].world, 48);
        hb[i].mesh = ctx->inst[i].mesh_id;
        hb[i].inst = i;
        hb[i].pad0 = hb[i].pad1 = 0u;
    }
    if ((rc = copy_staged(ctx, 5, ctx->d_refit_inst, sizeof(GpuInstBox) * (size_t)n, st)) != GKRT_OK) return rc;
    GK_CUDA(gpu_bvh_refit_instances(ctx->refit, ctx->d_refit_inst, ctx->d_blas_box, ctx->d_nodes, ctx->d_refit_ubox,
                                    ctx->d_refit_arrive, ctx->d_wide, ctx->tlas_wide_count, ctx->d_error, kErrRefit,
                                    st));
    ++ctx->tlas_refits;
    return GKRT_OK;
}

// The emissive-triangle table of the current instances (rebuilt with every instance update).
int build_emitters(GkrtContext* ctx, cudaStream_t st) {
    EmitterTable t;
    build_emitter_table(ctx->inst.data(), (uint32_t)ctx->inst.size(), ctx->meshes.data(), ctx->pos_host.data(),
                        ctx->idx_host.data(), ctx->slot_tris, ctx->mat_host.data(), ctx->nmat, t);
    const uint32_t n = (uint32_t)t.alias.size();
    if (n > ctx->emit_cap) {
        dfree(ctx->d_emit);
        dfree(ctx->d_emit_alias);
        ctx->emit_cap = 0;
        GK_CUDA(cudaMalloc((void**)&ctx->d_emit, (size_t)n * 5 * sizeof(float4)));
        GK_CUDA(cudaMalloc((void**)&ctx->d_emit_alias, (size_t)n * sizeof(float2)));
        ctx->emit_cap = n;
    }
    int rc;
    const size_t gb = t.geo.size() * sizeof(float4), ab = t.alias.size() * sizeof(float2);
    void* hg = stage_buf(ctx, 3, gb + 16);
    void* ha = stage_buf(ctx, 4, ab + 16);
    if (!hg || !ha) return fail(ctx, GKRT_ERR_OOM, "page-locked staging of the emitter table");
    if (gb) std::memcpy(hg, t.geo.data(), gb);
    if (ab) std::memcpy(ha, t.alias.data(), ab);
    if ((rc = copy_staged(ctx, 3, ctx->d_emit, gb, st)) != GKRT_OK) return rc;
    if ((rc = copy_staged(ctx, 4, ctx->d_emit_alias, ab, st)) != GKRT_OK) return rc;
    ctx->nemit = n;
    return GKRT_OK;
}

int ensure_bvh(GkrtContext* ctx, uint32_t flags, cudaStream_t st) {
    if (!ctx->has_scene) return fail(ctx, GKRT_ERR_STATE, "no scene uploaded");
    int rc;
    if ((flags & GKRT_BUILD_BLAS) || !ctx->blas_ready) {
        if ((rc = build_blas(ctx, st)) != GKRT_OK) return rc;
    }
    if ((flags & GKRT_BUILD_TLAS) || !ctx->tlas_ready) {
        if ((rc = build_tlas(ctx, st)) != GKRT_OK) return rc;
    }
    return GKRT_OK;
}

SceneView scene_view(GkrtContext* c) {
    SceneView S;
    S.nodes = c->d_nodes;
    S.wide = c->d_wide;
    S.tris = c->d_tris;
    S.inst = c->d_inst;
    S.tlas_root = c->tlas_root;
    S.tlas_wide_root = c->tlas_wide_root;
    S.error = c->d_error;
    S.node_count = (uint32_t)c->d_nodes_cap;
    S.wide_count = (uint32_t)c->d_wide_cap;
    S.tri_count = c->tri_count;
    S.inst_count = (uint32_t)c->inst.size();
    return S;
}

ShadeScene shade_scene(GkrtContext* ctx) {
    ShadeScene sc;
    sc.S = scene_view(ctx);
    sc.normals = ctx->d_nrm;
    sc.slots = ctx->d_slot;
    sc.indices = ctx->d_idx;
    sc.inst_mat = ctx->d_inst_mat;
    sc.inst_prev = ctx->d_inst_prev;
    sc.mats = ctx->d_mat;
    sc.nmat = ctx->nmat;
    sc.cubes = ctx->d_cubes;
    sc.voxels = ctx->d_voxels;
    sc.emit = ctx->d_emit;
    sc.emit_alias = ctx->d_emit_alias;
    sc.nemit = ctx->nemit;
    sc.tex = ctx->d_tex;
    sc.uv = ctx->d_uv;
    sc.tangents = ctx->d_tan;
    return sc;
}

// Texels of one channel byte as the sampler returns them: UNORM c / 255; sRGB through the
// sRGB transfer function (Vulkan's sRGB-to-linear conversion) evaluated in double.
float unorm8(uint8_t c) { return (float)c / 255.0f; }
float srgb8(uint8_t c) {
    const double v = (double)c / 255.0;
    return (float)(v <= 0.04045 ? v / 12.92 : std::pow((v + 0.055) / 1.055, 2.4));
}

// ProjectHdrToSh (Texture.cpp:180-254): the equirectangular image projected on the nine real
// spherical harmonics of bands 0-2, texel (x, y) at theta = (y + 1/2) pi / h, phi = (x + 1/2)
// 2 pi / w, direction (sin theta cos phi, cos theta, sin theta sin phi), weighted by its solid
// angle sin theta (pi / h)(2 pi / w), unnormalised. Accumulated in double in row-major texel
// order and rounded to float once (the reference sums in float).
void project_sky_sh(const float4* t, uint32_t w, uint32_t h, float out[27]) {
    const double pi = 3.14159265358979323846;
    const double c0 = 0.282095, c1 = 0.488603, c2 = 1.092548, c3 = 0.315392, c4 = 0.546274;
    double acc[27] = {0.0};
    std::vector<double> sp(w), cp(w);
    for (uint32_t x = 0; x < w; ++x) {
        const double phi = ((double)x + 0.5) / (double)w * (2.0 * pi);
        sp[x] = std::sin(phi);
        cp[x] = std::cos(phi);
    }
    for (uint32_t y = 0; y < h; ++y) {
        const double theta = ((double)y + 0.5) / (double)h * pi;
        const double st = std::sin(theta), ct = std::cos(theta);
        const double wt = st * (pi / (double)h) * (2.0 * pi / (double)w);
        for (uint32_t x = 0; x < w; ++x) {
            const double dx = st * cp[x], dy = ct, dz = st * sp[x];
            const double b[9] = {c0, -c1 * dy, c1 * dz, -c1 * dx, c2 * dx * dy, -c2 * dy * dz,
                                 c3 * (3.0 * dy * dy - 1.0), -c2 * dx * dz, c4 * (dx * dx - dz * dz)};
            const float4 v = t[(size_t)y * w + x];
            for (int i = 0; i < 9; ++i) {
                acc[i] += (double)v.x * b[i] * wt;
                acc[9 + i] += (double)v.y * b[i] * wt;
                acc[18 + i] += (double)v.z * b[i] * wt;
            }
        }
    }
    for (int k = 0; k < 27; ++k) out[k] = (float)acc[k];
}

int check_frame(GkrtContext* ctx, const GkrtFrameConstants* fc) {
    if (!ctx) return GKRT_ERR_INVALID_ARG;
    if (!fc) return fail(ctx, GKRT_ERR_INVALID_ARG, "null frame constants");
    if (ctx->W == 0 || ctx->H == 0) return fail(ctx, GKRT_ERR_STATE, "gkrt_resize was not called");
    return GKRT_OK;
}

}  // namespace

int gkrt_internal_fail(GkrtContext* ctx, int code, const std::string& msg) { return fail(ctx, code, msg); }

// cuTensorMapEncodeTiled through the runtime's driver entry point (no libcuda link needed).
cudaError_t gkrt_encode_tmap_2d(CUtensorMap* map, const void* base, uint32_t elems_x, uint32_t rows,
                                uint32_t row_bytes, uint32_t box_x, uint32_t box_y, bool is_float) {
    typedef CUresult (*EncodeFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
    static EncodeFn fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q);
        if (e != cudaSuccess) return e;
        if (q != cudaDriverEntryPointSuccess || !p) return cudaErrorNotSupported;
        fn = (EncodeFn)p;
    }
    if (((uintptr_t)base & 15u) || (row_bytes & 15u) || box_x == 0 || box_x > 256 || box_y == 0 || box_y > 256 ||
        ((box_x * 4u) & 15u))
        return cudaErrorInvalidValue;
    const cuuint64_t dims[2] = {elems_x, rows};
    const cuuint64_t strides[1] = {row_bytes};
    const cuuint32_t box[2] = {box_x, box_y};
    const cuuint32_t estr[2] = {1, 1};
    CUresult r = fn(map, is_float ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_UINT32, 2,
                    const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                    CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

// cuTensorMapEncodeTiled for bf16 tensors of rank 2..5; zeros outside the tensor. swizzle: 0
// none (dense boxes), 32, 64 or 128 bytes (the tensor-core kernels' operand layouts; the inner
// box at most that many bytes).
static cudaError_t encode_tmap_bf16(CUtensorMap* map, const void* base, uint32_t rank, const uint64_t* dims,
                                    const uint64_t* strides_bytes, const uint32_t* box, int swizzle) {
    typedef CUresult (*EncodeFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
    static EncodeFn fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q);
        if (e != cudaSuccess) return e;
        if (q != cudaDriverEntryPointSuccess || !p) return cudaErrorNotSupported;
        fn = (EncodeFn)p;
    }
    if (rank < 2 || rank > 5 || ((uintptr_t)base & 15u) || (box[0] * 2u) % 16u ||
        (swizzle != 0 && swizzle != 32 && swizzle != 64 && swizzle != 128) ||
        (swizzle && box[0] * 2u > (uint32_t)swizzle))
        return cudaErrorInvalidValue;
    cuuint64_t d[5], s[4];
    cuuint32_t b[5], es[5];
    for (uint32_t i = 0; i < rank; ++i) {
        d[i] = dims[i];
        b[i] = box[i];
        es[i] = 1;
        if (box[i] == 0 || box[i] > 256) return cudaErrorInvalidValue;
    }
    for (uint32_t i = 0; i + 1 < rank; ++i) {
        s[i] = strides_bytes[i];
        if (s[i] % 16u) return cudaErrorInvalidValue;
    }
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, rank, const_cast<void*>(base), d, s, b, es,
                    CU_TENSOR_MAP_INTERLEAVE_NONE,
                    swizzle == 128  ? CU_TENSOR_MAP_SWIZZLE_128B
                    : swizzle == 64 ? CU_TENSOR_MAP_SWIZZLE_64B
                    : swizzle == 32 ? CU_TENSOR_MAP_SWIZZLE_32B
                                    : CU_TENSOR_MAP_SWIZZLE_NONE,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

cudaError_t gkrt_encode_tmap_bf16(CUtensorMap* map, const void* base, uint32_t rank, const uint64_t* dims,
                                  const uint64_t* strides_bytes, const uint32_t* box) {
    return encode_tmap_bf16(map, base, rank, dims, strides_bytes, box, 64);
}
cudaError_t gkrt_encode_tmap_bf16_sw128(CUtensorMap* map, const void* base, uint32_t rank, const uint64_t* dims,
                                        const uint64_t* strides_bytes, const uint32_t* box) {
    return encode_tmap_bf16(map, base, rank, dims, strides_bytes, box, 128);
}
cudaError_t gkrt_encode_tmap_bf16_sw32(CUtensorMap* map, const void* base, uint32_t rank, const uint64_t* dims,
                                       const uint64_t* strides_bytes, const uint32_t* box) {
    return encode_tmap_bf16(map, base, rank, dims, strides_bytes, box, 32);
}
cudaError_t gkrt_encode_tmap_bf16_dense(CUtensorMap* map, const void* base, uint32_t rank, const uint64_t* dims,
                                        const uint64_t* strides_bytes, const uint32_t* box) {
    return encode_tmap_bf16(map, base, rank, dims, strides_bytes, box, 0);
}

int gkrt_internal_ready_view(GkrtContext* ctx, SceneView* view, unsigned long long** counters, int* device) {
    if (!ctx->has_scene || !ctx->blas_ready || !ctx->tlas_ready)
        return fail(ctx, GKRT_ERR_STATE, "scene and BVH must be built before this call (it allocates nothing)");
    *view = scene_view(ctx);
    *counters = ctx->d_counters;
    *device = ctx->device;
    return GKRT_OK;
}

extern "C" {

int gkrt_abi_version(void) { return GKRT_ABI_VERSION; }

int gkrt_context_create(const GkrtDeviceDesc* desc, GkrtContext** out) {
    if (!out) return GKRT_ERR_INVALID_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return GKRT_ERR_NO_DEVICE;
    }
    GkrtContext* ctx = new (std::nothrow) GkrtContext();
    if (!ctx) return GKRT_ERR_OOM;
    ctx->device = desc ? desc->device : 0;
    if (desc && desc->watchdog_ms) ctx->watchdog_ms = desc->watchdog_ms;
    if (ctx->device < 0 || ctx->device >= ndev || (desc && (desc->flags & ~GKRT_DEVICE_PASS_TIMERS))) {
        delete ctx;
        return GKRT_ERR_INVALID_ARG;
    }
    ctx->timers = desc && (desc->flags & GKRT_DEVICE_PASS_TIMERS);
    DeviceGuard device_guard(ctx->device);
    cudaError_t e = device_guard.status;
    for (int i = 0; i < kPassCount && ctx->timers && e == cudaSuccess; ++i)
        for (int k = 0; k < 2 && e == cudaSuccess; ++k) e = cudaEventCreate(&ctx->pass_ev[i][k]);
    if (e == cudaSuccess) e = cudaMalloc((void**)&ctx->d_counters, 8 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMalloc((void**)&ctx->d_error, sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc((void**)&ctx->d_work, sizeof(unsigned int));
    if (e == cudaSuccess) e = cudaMalloc((void**)&ctx->d_tex, GKRT_MAX_TEXTURES * sizeof(DevTex));
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, ctx->device);
    if (e == cudaSuccess) e = cudaMemset(ctx->d_counters, 0, 8 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(ctx->d_error, 0, sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemset(ctx->d_tex, 0, GKRT_MAX_TEXTURES * sizeof(DevTex));
    if (e != cudaSuccess) {
        dfree(ctx->d_counters);
        dfree(ctx->d_error);
        dfree(ctx->d_work);
        dfree(ctx->d_tex);
        for (auto& pe : ctx->pass_ev)
            for (cudaEvent_t& ev : pe)
                if (ev) cudaEventDestroy(ev);
        delete ctx;
        return e == cudaErrorMemoryAllocation ? GKRT_ERR_OOM : GKRT_ERR_CUDA;
    }
    *out = ctx;
    return GKRT_OK;
}

int gkrt_context_destroy(GkrtContext* ctx) {
    if (!ctx) return GKRT_ERR_INVALID_ARG;
    DeviceGuard device_guard(ctx->device);
    cudaDeviceSynchronize();
    free_images(ctx);
    free_scene(ctx);
    gkrt_unet_delete(ctx->unet);
    ctx->unet = nullptr;
    gpu_bvh_free(ctx->builder);
    ctx->builder = nullptr;
    dfree(ctx->d_output);
    for (StageSlot& S : ctx->stage)
        for (int k = 0; k < 2; ++k) {
            if (S.p[k]) cudaFreeHost(S.p[k]);
            if (S.ev[k]) cudaEventDestroy(S.ev[k]);
            S.p[k] = nullptr;
            S.ev[k] = nullptr;
        }
    dfree(ctx->d_counters);
    dfree(ctx->d_error);
    dfree(ctx->d_work);
    dfree(ctx->d_tex);
    for (float4*& t : ctx->tex_buf) dfree(t);
    for (auto& pe : ctx->pass_ev)
        for (cudaEvent_t& ev : pe)
            if (ev) cudaEventDestroy(ev);
    for (cudaEvent_t& ev : ctx->trace_ev)
        if (ev) cudaEventDestroy(ev);
    if (ctx->h_trace_counters) cudaFreeHost(ctx->h_trace_counters);
    delete ctx;
    return GKRT_OK;
}

const char* gkrt_last_error_message(const GkrtContext* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int gkrt_resize(GkrtContext* ctx, uint32_t width, uint32_t height) {
    if (!ctx) return GKRT_ERR_INVALID_ARG;
    if (width == 0 || height == 0 || width > 16384 || height > 16384)
        return fail(ctx, GKRT_ERR_INVALID_ARG, "image size must be 1..16384");
    DeviceGuard device_guard(ctx->device);
    free_images(ctx);
    const uint32_t pitch = (width + 3u) & ~3u;
    const size_t px = (size_t)pitch * height;
    for (int i = 0; i < GKRT_IMG_COUNT; ++i) {
        GK_CUDA(cudaMalloc(&ctx->img[i], px * image_bytes_per_px(i)));
        GK_CUDA(cudaMemset(ctx->img[i], 0, px * image_bytes_per_px(i)));
    }
    for (auto& t : ctx->atrous_tmp) {
        GK_CUDA(cudaMalloc((void**)&t, px * sizeof(float4)));
        GK_CUDA(cudaMemset(t, 0, px * sizeof(float4)));
    }
    ctx->W = width;
    ctx->H = height;
    ctx->P = pitch;
    return GKRT_OK;
}

int gkrt_scene_upload(GkrtContext* ctx, const GkrtSceneDesc* d) {
    if (!ctx) return GKRT_ERR_INVALID_ARG;
    if (!d) return fail(ctx, GKRT_ERR_INVALID_ARG, "null scene");
    if ((d->vertex_count && (!d->positions || !d->normals || !d->material_slots)) ||
        (d->index_count && !d->indices) || (d->mesh_count && !d->meshes) || (d->material_count == 0) ||
        !d->materials || (d->instance_count && !d->instances) || (d->light_count && !d->lights))
        return fail(ctx, GKRT_ERR_INVALID_ARG, "scene arrays missing for non-zero counts");
    if (d->instance_count > (1u << 24)) return fail(ctx, GKRT_ERR_DEVICE_LIMIT, "too many instances");
    if ((uint64_t)d->index_count / 3 >= (1u << 28)) return fail(ctx, GKRT_ERR_DEVICE_LIMIT, "too many triangles");
    for (uint32_t i = 0; i < d->vertex_count; ++i)
        if (!finite3(d->positions + 4 * (size_t)i) || !finite3(d->normals + 4 * (size_t)i))
            return fail(ctx, GKRT_ERR_INVALID_ARG, "non-finite vertex position or normal");
    for (uint32_t i = 0; i < d->vertex_count; ++i)
        if (d->material_slots[i] > 15u) return fail(ctx, GKRT_ERR_INVALID_ARG, "material slot above 15");
    for (uint32_t m = 0; m < d->mesh_count; ++m) {
        const GkrtMesh& ms = d->meshes[m];
        if (ms.index_count % 3 != 0) return fail(ctx, GKRT_ERR_INVALID_ARG, "mesh index_count not a multiple of 3");
        if ((uint64_t)ms.index_offset + ms.index_count > d->index_count)
            return fail(ctx, GKRT_ERR_INVALID_ARG, "mesh index range outside the index buffer");
        if ((uint64_t)ms.vertex_offset + ms.vertex_count > d->vertex_count)
            return fail(ctx, GKRT_ERR_INVALID_ARG, "mesh vertex range outside the vertex buffer");
        for (uint32_t k = 0; k < ms.index_count; ++k)
            if (d->indices[ms.index_offset + k] >= ms.vertex_count)
                return fail(ctx, GKRT_ERR_INVALID_ARG, "index outside its mesh's vertex range");
    }
    bool textured = false;
    for (uint32_t i = 0; i < d->material_count; ++i) {
        const GkrtMaterial& mt = d->materials[i];
        for (int32_t id : {mt.diffuse_texture_id, mt.mra_texture_id, mt.normal_texture_id}) {
            if (id < -1 || id >= (int32_t)GKRT_MAX_TEXTURES)
                return fail(ctx, GKRT_ERR_INVALID_ARG, "texture id outside -1 .. GKRT_MAX_TEXTURES - 1");
            textured = textured || id >= 0;
        }
        if (mt.material_model > GKRT_MAT_MIXTURE) return fail(ctx, GKRT_ERR_INVALID_ARG, "unknown material model");
    }
    for (uint32_t i = 0; d->texcoords && i < d->vertex_count; ++i)
        if (!std::isfinite(d->texcoords[2 * (size_t)i]) || !std::isfinite(d->texcoords[2 * (size_t)i + 1]))
            return fail(ctx, GKRT_ERR_INVALID_ARG, "non-finite texture coordinate");
    for (uint32_t i = 0; d->tangents && i < d->vertex_count; ++i)
        if (!finite3(d->tangents + 4 * (size_t)i) || !std::isfinite(d->tangents[4 * (size_t)i + 3]))
            return fail(ctx, GKRT_ERR_INVALID_ARG, "non-finite tangent");
    int rc = validate_instances(ctx, d->instances, d->instance_count, d->mesh_count, d->material_count);
    if (rc != GKRT_OK) return rc;
    DeviceGuard device_guard(ctx->device);
    free_scene(ctx);
    ctx->meshes.assign(d->meshes, d->meshes + d->mesh_count);
    ctx->inst.assign(d->instances, d->instances + d->instance_count);
    ctx->pos_host.assign(d->positions, d->positions + 4 * (size_t)d->vertex_count);
    ctx->idx_host.assign(d->indices, d->indices + d->index_count);
    ctx->nvert = d->vertex_count;
    ctx->nidx = d->index_count;
    ctx->nmat = d->material_count;
    ctx->mat_host.assign(d->materials, d->materials + d->material_count);
    if (d->light_count) ctx->lights_host.assign(d->lights, d->lights + d->light_count);
    mesh_slot_triangles(d->meshes, d->mesh_count, d->indices, d->material_slots, ctx->slot_tris);
    if ((rc = upload(ctx, ctx->d_pos, d->positions, 16 * (size_t)d->vertex_count)) != GKRT_OK) return rc;
    if ((rc = upload(ctx, ctx->d_nrm, d->normals, 16 * (size_t)d->vertex_count)) != GKRT_OK) return rc;
    if (d->texcoords && (rc = upload(ctx, ctx->d_uv, d->texcoords, 8 * (size_t)d->vertex_count)) != GKRT_OK) return rc;
    if (d->tangents && (rc = upload(ctx, ctx->d_tan, d->tangents, 16 * (size_t)d->vertex_count)) != GKRT_OK) return rc;
    ctx->textured = textured;
    if ((rc = upload(ctx, ctx->d_slot, d->material_slots, 4 * (size_t)d->vertex_count)) != GKRT_OK) return rc;
    if ((rc = upload(ctx, ctx->d_idx, d->indices, 4 * (size_t)d->index_count)) != GKRT_OK) return rc;
    if ((rc = upload(ctx, ctx->d_mat, d->materials, sizeof(GkrtMaterial) * (size_t)d->material_count)) != GKRT_OK)
        return rc;
    if (d->probe_cubes && d->probe_voxels) {
        const size_t n = (size_t)192 * 192 * 48;
        if ((rc = upload(ctx, ctx->d_cubes, d->probe_cubes, n * 14 * 4)) != GKRT_OK) return rc;
        if ((rc = upload(ctx, ctx->d_voxels, d->probe_voxels, n * 4 * 4)) != GKRT_OK) return rc;
    }
    ctx->has_scene = true;
    if ((rc = ensure_bvh(ctx, GKRT_BUILD_ALL, (cudaStream_t)0)) != GKRT_OK) return rc;
    if ((rc = build_emitters(ctx, (cudaStream_t)0)) != GKRT_OK) return rc;
    GK_CUDA(cudaStreamSynchronize((cudaStream_t)0));
    return GKRT_OK;
}

int gkrt_scene_update_instances(GkrtContext* ctx, const GkrtInstance* instances, uint32_t count, void* stream) {
    if (!ctx) return GKRT_ERR_INVALID_ARG;
    if (!ctx->has_scene) return fail(ctx, GKRT_ERR_STATE, "no scene uploaded");
    if (!instances || count != ctx->inst.size())
        return fail(ctx, GKRT_ERR_INVALID_ARG, "instance update must keep the instance count");
    int rc = validate_instances(ctx, instances, count, (uint32_t)ctx->meshes.size(), ctx->nmat);
    if (rc != GKRT_OK) return rc;
    DeviceGuard device_guard(ctx->device);
    const PassScope scope(ctx, kPassTlas, (cudaStream_t)stream);
    ctx->inst.assign(instances, instances + count);
    // host work first (the instance tables inside build_tlas), uploaded asynchronously, so that
    // it overlaps the stream's earlier frames; the emitter table is built on the host while the
    // GPU builds the instance level
    if (!ctx->blas_ready) {
        if ((rc = build_emitters(ctx, (cudaStream_t)stream)) != GKRT_OK) return rc;
        return ensure_bvh(ctx, 0, (cudaStream_t)stream);
    }
    return build_tlas(ctx, (cudaStream_t)stream, build_emitters);
}

int gkrt_scene_refit_instances(GkrtContext* ctx, const GkrtInstance* instances, uint32_t count, void* stream) {
    if (!ctx) return GKRT_ERR_INVALID_ARG;
    if (!ctx->has_scene) return fail(ctx, GKRT_ERR_STATE, "no scene uploaded");
    if (!instances || count != ctx->inst.size())
        return fail(ctx, GKRT_ERR_INVALID_ARG, "instance update must keep the instance count");
    int rc = validate_instances(ctx, instances, count, (uint32_t)ctx->meshes.size(), ctx->nmat);
    if (rc != GKRT_OK) return rc;
    DeviceGuard device_guard(ctx->device);
    const PassScope scope(ctx, kPassTlas, (cudaStream_t)stream);
    ctx->inst.assign(instances, instances + count);
    if ((rc = build_emitters(ctx, (cudaStream_t)stream)) != GKRT_OK) return rc;
    if (!ctx->blas_ready || !ctx->tlas_ready) return ensure_bvh(ctx, 0, (cudaStream_t)stream);
    std::vector<uint8_t> m;
    tlas_members(ctx, m);
    if (m != ctx->tlas_members) return build_tlas(ctx, (cudaStream_t)stream);   // the tree's members changed
    return refit_tlas(ctx, (cudaStream_t)stream);
}

// The newest trace pass whose counters have reached the host (without waiting): node visits
// per ray into visits_last, and into visits_base when none is set and the pass came after the
// last rebuild.
static void poll_trace_counters(GkrtContext* ctx) {
    if (!ctx->h_trace_counters) return;
    for (uint64_t back = 1; back <= 2 && back <= ctx->trace_seq; ++back) {
        const uint64_t seq = ctx->trace_seq - back;
        if (seq < ctx->trace_seq_read) break;
        if (cudaEventQuery(ctx->trace_ev[seq & 1]) != cudaSuccess) continue;
        const unsigned long long* c = ctx->h_trace_counters + 7 * (seq & 1);
        if (c[0] > 0) {
            ctx->visits_last = (double)c[3] / (double)c[0];
            if (ctx->visits_base < 0.0 && seq >= ctx->base_after) ctx->visits_base = ctx->visits_last;
        }
        ctx->trace_seq_read = seq + 1;
        break;
    }
    cudaGetLastError();   // a not-ready query leaves no error behind
}

int gkrt_scene_update_instances_auto(GkrtContext* ctx, const GkrtInstance* instances, uint32_t count,
                                     float growth_limit, void* stream) {
    if (!ctx) return GKRT_ERR_INVALID_ARG;
    if (!(growth_limit >= 1.0f) || !std::isfinite(growth_limit))
        return fail(ctx, GKRT_ERR_INVALID_ARG, "growth_limit must be a finite number >= 1");
    if (!ctx->has_scene) return fail(ctx, GKRT_ERR_STATE, "no scene uploaded");
    if (!instances || count != ctx->inst.size())
        return fail(ctx, GKRT_ERR_INVALID_ARG, "instance update must keep the instance count");
    int rc = validate_instances(ctx, instances, count, (uint32_t)ctx->meshes.size(), ctx->nmat);
    if (rc != GKRT_OK) return rc;
    DeviceGuard device_guard(ctx->device);
    if (!ctx->h_trace_counters) {   // first use: trace passes start recording their counters
        for (cudaEvent_t& ev : ctx->trace_ev)
            if (!ev) GK_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        GK_CUDA(cudaMallocHost((void**)&ctx->h_trace_counters, 14 * sizeof(unsigned long long)));
    }
    const PassScope scope(ctx, kPassTlas, (cudaStream_t)stream);
    cudaStream_t st = (cudaStream_t)stream;
    ctx->inst.assign(instances, instances + count);
    poll_trace_counters(ctx);
    bool refit = ctx->blas_ready && ctx->tlas_ready;
    if (refit) {
        std::vector<uint8_t> m;
        tlas_members(ctx, m);
        refit = m == ctx->tlas_members;
    }
    if (refit && ctx->visits_base > 0.0 && ctx->visits_last > 0.0)
        refit = ctx->visits_last < (double)growth_limit * ctx->visits_base;
    if (refit) {
        if ((rc = build_emitters(ctx, st)) != GKRT_OK) return rc;
        return refit_tlas(ctx, st);
    }
    // rebuild: the next completed pass traced on the new tree sets the baseline
    ctx->visits_base = -1.0;
    ctx->base_after = ctx->trace_seq;
    if (!ctx->blas_ready) {
        if ((rc = build_emitters(ctx, st)) != GKRT_OK) return rc;
        return ensure_bvh(ctx, 0, st);
    }
    return build_tlas(ctx, st, build_emitters);
}

int gkrt_build_bvh(GkrtContext* ctx, uint32_t flags, void* stream) {
    if (!ctx) return GKRT_ERR_INVALID_ARG;
    if (flags & ~(GKRT_BUILD_ALL | GKRT_BUILD_ON_HOST)) return fail(ctx, GKRT_ERR_INVALID_ARG, "unknown build flags");
    DeviceGuard device_guard(ctx->device);
    const bool host = (flags & GKRT_BUILD_ON_HOST) != 0;
    if (host != ctx->host_build) {
        ctx->host_build = host;
        flags |= GKRT_BUILD_ALL;   // both levels come from the same builder
    }
    return ensure_bvh(ctx, flags, (cudaStream_t)stream);
}

int gkrt_trace_pass(GkrtContext* ctx, const GkrtFrameConstants* fc, void* stream) {
    int rc = check_frame(ctx, fc);
    if (rc != GKRT_OK) return rc;
    if (!ctx->has_scene) return fail(ctx, GKRT_ERR_STATE, "no scene uploaded");
    if (fc->nee_mode > GKRT_NEE_EMISSIVE) return fail(ctx, GKRT_ERR_INVALID_ARG, "unknown nee_mode");
    if ((fc->flags & GKRT_FRAME_SKY_TEXTURE) && fc->sky_index >= GKRT_MAX_TEXTURES)
        return fail(ctx, GKRT_ERR_INVALID_ARG, "sky_index outside the texture pool");
    DeviceGuard device_guard(ctx->device);
    cudaStream_t st = (cudaStream_t)stream;
    if ((rc = ensure_bvh(ctx, 0, st)) != GKRT_OK) return rc;
    const PassScope scope(ctx, kPassRt, st);
    const ShadeScene sc = shade_scene(ctx);
    PixelImages im;
    im.single_diffuse = (float4*)ctx->img[GKRT_IMG_SINGLE_DIFFUSE];
    im.single_specular = (float4*)ctx->img[GKRT_IMG_SINGLE_SPECULAR];
    im.albedo = (float4*)ctx->img[GKRT_IMG_ALBEDO];
    im.normal = (float4*)ctx->img[GKRT_IMG_NORMAL];
    im.object_id = (uint32_t*)ctx->img[GKRT_IMG_OBJECT_ID];
    im.motion = (float2*)ctx->img[GKRT_IMG_MOTION];
    im.prev_depth = (float*)ctx->img[GKRT_IMG_PREV_DEPTH];
    im.motion_moment = (uint32_t*)ctx->img[GKRT_IMG_MOTION_MOMENT];
    im.hit_inst = (uint32_t*)ctx->img[GKRT_IMG_HIT_INST];
    im.hit_prim = (uint32_t*)ctx->img[GKRT_IMG_HIT_PRIM];
    GK_CUDA(cudaMemsetAsync(ctx->d_counters, 0, 6 * sizeof(unsigned long long), st));
    // the stack bound check_stack_bound enforced at build time, at least 8 entries
    const int stack_words = std::max(8, std::min(kStackSize, ctx->blas_bin_depth + ctx->tlas_bin_depth + 3));
    GK_CUDA(gkrt_launch_trace_pass(sc, *fc, (int)ctx->W, (int)ctx->H, (int)ctx->P, im, ctx->d_counters, ctx->d_work,
                                   ctx->num_sms, stack_words, ctx->textured, st));
    if (ctx->h_trace_counters) {   // the refit-or-rebuild policy is in use: this pass's counters
        const int k = (int)(ctx->trace_seq & 1);
        GK_CUDA(cudaMemcpyAsync(ctx->h_trace_counters + 7 * k, ctx->d_counters, 7 * sizeof(unsigned long long),
                                cudaMemcpyDeviceToHost, st));
        GK_CUDA(cudaEventRecord(ctx->trace_ev[k], st));
        ++ctx->trace_seq;
    }
    return GKRT_OK;
}

int gkrt_texture_upload(GkrtContext* ctx, uint32_t texture_id, uint32_t width, uint32_t height, uint32_t format,
                        const void* texels, size_t bytes) {
    if (!ctx) return GKRT_ERR_INVALID_ARG;
    if (texture_id >= GKRT_MAX_TEXTURES) return fail(ctx, GKRT_ERR_INVALID_ARG, "texture id >= GKRT_MAX_TEXTURES");
    if (format > GKRT_TEX_RGBA32F) return fail(ctx, GKRT_ERR_INVALID_ARG, "unknown texture format");
    if (width == 0 || height == 0 || width > 16384 || height > 16384)
        return fail(ctx, GKRT_ERR_INVALID_ARG, "texture size must be 1..16384");
    const size_t n = (size_t)width * height;
    if (!texels || bytes != n * (format == GKRT_TEX_RGBA32F ? 16u : 4u))
        return fail(ctx, GKRT_ERR_INVALID_ARG, "texel buffer missing or of the wrong size");
    std::vector<float4> t(n);
    if (format == GKRT_TEX_RGBA32F) {
        std::memcpy(t.data(), texels, n * 16);
    } else {
        const uint8_t* b = static_cast<const uint8_t*>(texels);
        for (size_t i = 0; i < n; ++i) {
            const uint8_t* c = b + 4 * i;
            if (format == GKRT_TEX_RGBA8_SRGB) t[i] = make_float4(srgb8(c[0]), srgb8(c[1]), srgb8(c[2]), unorm8(c[3]));
            else t[i] = make_float4(unorm8(c[0]), unorm8(c[1]), unorm8(c[2]), unorm8(c[3]));
        }
    }
    DeviceGuard device_guard(ctx->device);
    if (ctx->tex_buf.size() < GKRT_MAX_TEXTURES) ctx->tex_buf.resize(GKRT_MAX_TEXTURES, nullptr);
    float4* d = nullptr;
    GK_CUDA(cudaMalloc((void**)&d, n * sizeof(float4)));
    cudaError_t e = cudaMemcpy(d, t.data(), n * sizeof(float4), cudaMemcpyHostToDevice);
    DevTex entry;
    entry.texels = d;
    entry.w = width;
    entry.h = height;
    if (e == cudaSuccess) e = cudaDeviceSynchronize();   // no kernel still reads the texture replaced here
    if (e == cudaSuccess) e = cudaMemcpy(ctx->d_tex + texture_id, &entry, sizeof(DevTex), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(d);
        return cuda_fail(ctx, e, "gkrt_texture_upload");
    }
    dfree(ctx->tex_buf[texture_id]);
    ctx->tex_buf[texture_id] = d;
    if (format == GKRT_TEX_RGBA32F || !ctx->tex_sh.empty()) {
        if (ctx->tex_sh.empty()) ctx->tex_sh.assign((size_t)GKRT_MAX_TEXTURES * 27u, 0.0f);
        float* c = ctx->tex_sh.data() + (size_t)texture_id * 27u;
        if (format == GKRT_TEX_RGBA32F) project_sky_sh(t.data(), width, height, c);
        else std::fill(c, c + 27, 0.0f);
    }
    return GKRT_OK;
}

int gkrt_reproject_pass(GkrtContext* ctx, const GkrtFrameConstants* fc, void* stream) {
    int rc = check_frame(ctx, fc);
    if (rc != GKRT_OK) return rc;
    DeviceGuard device_guard(ctx->device);
    const PassScope scope(ctx, kPassReproject, (cudaStream_t)stream);
    ReprojectArgs a;
    a.W = (int)ctx->W; a.H = (int)ctx->H; a.P = (int)ctx->P;
    a.err = ctx->d_error;
    a.progressive = fc->progressive_render;
    a.temporal_frames = fc->temporal_frames;
    a.src_d = (const float4*)ctx->img[GKRT_IMG_SINGLE_DIFFUSE];
    a.src_s = (const float4*)ctx->img[GKRT_IMG_SINGLE_SPECULAR];
    a.src_a = (const float4*)ctx->img[GKRT_IMG_ALBEDO];
    a.prev_d = (const float4*)ctx->img[GKRT_IMG_PREV_DIFFUSE];
    a.prev_s = (const float4*)ctx->img[GKRT_IMG_PREV_SPECULAR];
    a.prev_a = (const float4*)ctx->img[GKRT_IMG_PREV_ALBEDO];
    a.normal = (const float4*)ctx->img[GKRT_IMG_NORMAL];
    a.motion = (const float2*)ctx->img[GKRT_IMG_MOTION];
    a.id0 = (const uint32_t*)ctx->img[GKRT_IMG_OBJECT_ID];
    a.id1 = (const uint32_t*)ctx->img[GKRT_IMG_OBJECT_ID_PREV];
    a.moment = (const uint32_t*)ctx->img[GKRT_IMG_MOTION_MOMENT];
    a.acc_d = (float4*)ctx->img[GKRT_IMG_ACCUM_DIFFUSE];
    a.acc_s = (float4*)ctx->img[GKRT_IMG_ACCUM_SPECULAR];
    a.acc_a = (float4*)ctx->img[GKRT_IMG_ACCUM_ALBEDO];
    GK_CUDA(gkrt_launch_reproject(a, (cudaStream_t)stream));
    return GKRT_OK;
}

int gkrt_denoise_pass(GkrtContext* ctx, const GkrtFrameConstants* fc, void* stream) {
    int rc = check_frame(ctx, fc);
    if (rc != GKRT_OK) return rc;
    if (fc->denoiser > GKRT_DENOISE_UNET) return fail(ctx, GKRT_ERR_UNSUPPORTED, "unknown denoiser");
    DeviceGuard device_guard(ctx->device);
    const PassScope scope(ctx, kPassCompose, (cudaStream_t)stream);
    if (fc->denoiser == GKRT_DENOISE_UNET) {
        if (!ctx->unet) return fail(ctx, GKRT_ERR_STATE, "gkrt_unet_init was not called");
        if (ctx->W % 8 || ctx->H % 8) return fail(ctx, GKRT_ERR_UNSUPPORTED, "the learned denoiser needs sizes divisible by 8");
        cudaStream_t st = (cudaStream_t)stream;
        GK_CUDA(gkrt_unet_denoise_frame(ctx->unet, (const float4*)ctx->img[GKRT_IMG_SINGLE_DIFFUSE],
                                        (const float4*)ctx->img[GKRT_IMG_SINGLE_SPECULAR],
                                        (const float4*)ctx->img[GKRT_IMG_ALBEDO], (const float4*)ctx->img[GKRT_IMG_NORMAL],
                                        (const float*)ctx->img[GKRT_IMG_PREV_DEPTH], (int)ctx->W, (int)ctx->H,
                                        (int)ctx->P, nullptr, st));
        ComposeArgs a;
        a.W = (int)ctx->W; a.H = (int)ctx->H; a.P = (int)ctx->P;
        a.bf_size = 0; a.hdr = fc->hdr;
        a.bf_sigma = 0.0f; a.bf_sigma_lum = 0.0f; a.paper_white_nit = fc->paper_white_nit; a.pad = 0.0f;
        a.err = ctx->d_error;
        a.acc_d = a.acc_s = a.acc_a = nullptr;
        a.out = (float4*)ctx->img[GKRT_IMG_DENOISED];
        a.out_linear = (float4*)ctx->img[GKRT_IMG_DENOISED_LINEAR];
        GK_CUDA(gkrt_launch_unet_compose(a, gkrt_unet_output(ctx->unet), st));
        return GKRT_OK;
    }
    if (fc->denoiser == GKRT_DENOISE_ATROUS && fc->bf_size > 0u) {
        AtrousArgs a;
        a.W = (int)ctx->W; a.H = (int)ctx->H; a.P = (int)ctx->P;
        a.step = 1; a.last = 0; a.hdr = fc->hdr;
        a.sigma_lum = fc->bf_sigma_lum;
        a.paper_white_nit = fc->paper_white_nit;
        a.err = ctx->d_error;
        a.normal = (const float4*)ctx->img[GKRT_IMG_NORMAL];
        a.albedo = (const float4*)ctx->img[GKRT_IMG_ACCUM_ALBEDO];
        a.spec = (const float4*)ctx->img[GKRT_IMG_ACCUM_SPECULAR];
        a.id0 = (const uint32_t*)ctx->img[GKRT_IMG_OBJECT_ID];
        a.out = nullptr;
        a.final_out = (float4*)ctx->img[GKRT_IMG_DENOISED];
        a.final_linear = (float4*)ctx->img[GKRT_IMG_DENOISED_LINEAR];
        GK_CUDA(gkrt_launch_atrous(a, (const float4*)ctx->img[GKRT_IMG_ACCUM_DIFFUSE], ctx->atrous_tmp[0],
                                   ctx->atrous_tmp[1], (cudaStream_t)stream));
        return GKRT_OK;
    }
    ComposeArgs a;
    a.W = (int)ctx->W; a.H = (int)ctx->H; a.P = (int)ctx->P;
    a.bf_size = fc->bf_size;
    a.hdr = fc->hdr;
    a.bf_sigma = fc->bf_sigma;
    a.bf_sigma_lum = fc->bf_sigma_lum;
    a.paper_white_nit = fc->paper_white_nit;
    a.pad = 0.0f;
    a.err = ctx->d_error;
    a.acc_d = (const float4*)ctx->img[GKRT_IMG_ACCUM_DIFFUSE];
    a.acc_s = (const float4*)ctx->img[GKRT_IMG_ACCUM_SPECULAR];
    a.acc_a = (const float4*)ctx->img[GKRT_IMG_ACCUM_ALBEDO];
    a.out = (float4*)ctx->img[GKRT_IMG_DENOISED];
    a.out_linear = (float4*)ctx->img[GKRT_IMG_DENOISED_LINEAR];
    GK_CUDA(gkrt_launch_compose(a, (cudaStream_t)stream));
    return GKRT_OK;
}

int gkrt_end_frame(GkrtContext* ctx, void* stream) {
    if (!ctx) return GKRT_ERR_INVALID_ARG;
    if (ctx->W == 0) return fail(ctx, GKRT_ERR_STATE, "gkrt_resize was not called");
    DeviceGuard device_guard(ctx->device);
    const PassScope scope(ctx, kPassCopy, (cudaStream_t)stream);   // a buffer swap: no GPU work
    const int pairs[4][2] = {{GKRT_IMG_ACCUM_DIFFUSE, GKRT_IMG_PREV_DIFFUSE},
                             {GKRT_IMG_ACCUM_SPECULAR, GKRT_IMG_PREV_SPECULAR},
                             {GKRT_IMG_ACCUM_ALBEDO, GKRT_IMG_PREV_ALBEDO},
                             {GKRT_IMG_OBJECT_ID, GKRT_IMG_OBJECT_ID_PREV}};
    for (auto& p : pairs) std::swap(ctx->img[p[0]], ctx->img[p[1]]);
    return GKRT_OK;
}

int gkrt_render_frame(GkrtContext* ctx, const GkrtFrameConstants* fc, void* stream) {
    if (!ctx) return GKRT_ERR_INVALID_ARG;
    DeviceGuard device_guard(ctx->device);
    int rc;
    if ((rc = gkrt_trace_pass(ctx, fc, stream)) != GKRT_OK) return rc;
    if ((rc = gkrt_reproject_pass(ctx, fc, stream)) != GKRT_OK) return rc;
    if ((rc = gkrt_denoise_pass(ctx, fc, stream)) != GKRT_OK) return rc;
    return gkrt_end_frame(ctx, stream);
}

int gkrt_get_pass_times(GkrtContext* ctx, GkrtPassTimes* out) {
    if (!ctx || !out) return GKRT_ERR_INVALID_ARG;
    if (!ctx->timers) return fail(ctx, GKRT_ERR_STATE, "the context was created without GKRT_DEVICE_PASS_TIMERS");
    DeviceGuard device_guard(ctx->device);
    float ms[kPassCount];
    for (int i = 0; i < kPassCount; ++i) {
        ms[i] = -1.0f;
        if (!ctx->pass_recorded[i]) continue;
        GK_CUDA(cudaEventSynchronize(ctx->pass_ev[i][1]));
        GK_CUDA(cudaEventElapsedTime(&ms[i], ctx->pass_ev[i][0], ctx->pass_ev[i][1]));
    }
    out->rt_pass_ms = ms[kPassRt];
    out->reproject_pass_ms = ms[kPassReproject];
    out->compose_pass_ms = ms[kPassCompose];
    out->copy_pass_ms = ms[kPassCopy];
    out->tlas_update_ms = ms[kPassTlas];
    out->reserved[0] = out->reserved[1] = out->reserved[2] = 0.0f;
    return GKRT_OK;
}

int gkrt_get_image(GkrtContext* ctx, int id, GkrtImageView* out) {
    if (!ctx || !out) return GKRT_ERR_INVALID_ARG;
    if (id < 0 || id >= GKRT_IMG_COUNT) return fail(ctx, GKRT_ERR_INVALID_ARG, "unknown image id");
    if (ctx->W == 0) return fail(ctx, GKRT_ERR_STATE, "gkrt_resize was not called");
    out->device_ptr = ctx->img[id];
    out->width = ctx->W;
    out->height = ctx->H;
    out->pitch_bytes = (uint32_t)(ctx->P * image_bytes_per_px(id));
    out->format = image_format(id);
    return GKRT_OK;
}

int gkrt_synchronize(GkrtContext* ctx, void* stream) {
    if (!ctx) return GKRT_ERR_INVALID_ARG;
    DeviceGuard device_guard(ctx->device);
    cudaStream_t st = (cudaStream_t)stream;
    auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        cudaError_t e = cudaStreamQuery(st);
        if (e == cudaSuccess) break;
        if (e != cudaErrorNotReady) return cuda_fail(ctx, e, "cudaStreamQuery");
        auto ms = std::chrono::duration_cast<std::chrono::milliseconds>(std::chrono::steady_clock::now() - t0).count();
        if ((uint64_t)ms > ctx->watchdog_ms) return fail(ctx, GKRT_ERR_TIMEOUT, "stream did not drain before the watchdog");
        std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
    uint32_t errw = 0;
    GK_CUDA(cudaMemcpy(&errw, ctx->d_error, 4, cudaMemcpyDeviceToHost));
    if (errw) {
        cudaMemset(ctx->d_error, 0, 4);
        return fail(ctx, GKRT_ERR_DEVICE_LIMIT,
                    (errw & kErrStack) ? "traversal stack overflow"
                    : (errw & kErrIter) ? "traversal iteration cap reached"
                                        : "a tile load did not complete within its wait limit");
    }
    return GKRT_OK;
}

int gkrt_copy_image_to_host(GkrtContext* ctx, int id, void* dst, size_t dst_bytes, void* stream) {
    GkrtImageView v;
    int rc = gkrt_get_image(ctx, id, &v);
    if (rc != GKRT_OK) return rc;
    const size_t row = (size_t)v.width * image_bytes_per_px(id);
    if (!dst || dst_bytes < row * v.height) return fail(ctx, GKRT_ERR_INVALID_ARG, "destination smaller than the image");
    DeviceGuard device_guard(ctx->device);
    // the host copy is dense (width x height); the device rows are padded
    GK_CUDA(cudaMemcpy2DAsync(dst, row, v.device_ptr, v.pitch_bytes, row, v.height, cudaMemcpyDeviceToHost,
                              (cudaStream_t)stream));
    return gkrt_synchronize(ctx, stream);
}

int gkrt_copy_image_to_host_async(GkrtContext* ctx, int id, void* dst, size_t dst_bytes, void* stream) {
    GkrtImageView v;
    int rc = gkrt_get_image(ctx, id, &v);
    if (rc != GKRT_OK) return rc;
    const size_t row = (size_t)v.width * image_bytes_per_px(id);
    if (!dst || dst_bytes < row * v.height) return fail(ctx, GKRT_ERR_INVALID_ARG, "destination smaller than the image");
    DeviceGuard device_guard(ctx->device);
    GK_CUDA(cudaMemcpy2DAsync(dst, row, v.device_ptr, v.pitch_bytes, row, v.height, cudaMemcpyDeviceToHost,
                              (cudaStream_t)stream));
    return GKRT_OK;
}

int gkrt_output_resize(GkrtContext* ctx, uint32_t width, uint32_t height) {
    if (!ctx) return GKRT_ERR_INVALID_ARG;
    if ((width == 0) != (height == 0) || width > 16384 || height > 16384)
        return fail(ctx, GKRT_ERR_INVALID_ARG, "output size must be 1..16384 (or 0 x 0 to free)");
    DeviceGuard device_guard(ctx->device);
    GK_CUDA(cudaDeviceSynchronize());
    dfree(ctx->d_output);
    ctx->OW = ctx->OH = 0;
    if (width == 0) return GKRT_OK;
    const size_t bytes = (size_t)width * height * 4;
    GK_CUDA(cudaMalloc((void**)&ctx->d_output, bytes));
    GK_CUDA(cudaMemset(ctx->d_output, 0, bytes));
    ctx->OW = width;
    ctx->OH = height;
    return GKRT_OK;
}

int gkrt_output_pass(GkrtContext* ctx, const GkrtOutputDesc* d, void* stream) {
    if (!ctx || !d) return GKRT_ERR_INVALID_ARG;
    if (!ctx->d_output) return fail(ctx, GKRT_ERR_STATE, "gkrt_output_resize was not called");
    if (ctx->W == 0) return fail(ctx, GKRT_ERR_STATE, "gkrt_resize was not called");
    if (d->mode != GKRT_OUTPUT_RESOLVE && d->mode != GKRT_OUTPUT_FSR)
        return fail(ctx, GKRT_ERR_INVALID_ARG, "unknown output mode");
    if (d->source_image >= GKRT_IMG_COUNT || image_format((int)d->source_image) != GKRT_FMT_F32X4)
        return fail(ctx, GKRT_ERR_INVALID_ARG, "output source must be an RGBA32F image");
    if (d->width == 0 || d->height == 0 || d->width > 65536 || d->height > 65536)
        return fail(ctx, GKRT_ERR_INVALID_ARG, "output rectangle must be 1..65536 a side");
    if (std::abs((long long)d->offset_x) > 65536 || std::abs((long long)d->offset_y) > 65536)
        return fail(ctx, GKRT_ERR_INVALID_ARG, "output offset beyond +-65536");
    DeviceGuard device_guard(ctx->device);
    const float4* src = static_cast<const float4*>(ctx->img[d->source_image]);
    const cudaStream_t st = (cudaStream_t)stream;
    if (d->mode == GKRT_OUTPUT_RESOLVE)
        GK_CUDA(gkrt_launch_output_resolve(src, (int)ctx->W, (int)ctx->H, (int)ctx->P, ctx->d_output, (int)ctx->OW,
                                           (int)ctx->OH, d->offset_x, d->offset_y, (int)d->width, (int)d->height, st));
    else
        GK_CUDA(gkrt_launch_output_fsr(src, (int)ctx->W, (int)ctx->H, (int)ctx->P, ctx->d_output, (int)ctx->OW,
                                       (int)ctx->OH, d->offset_x, d->offset_y, (int)d->width, (int)d->height, st));
    return GKRT_OK;
}

int gkrt_get_output(GkrtContext* ctx, GkrtImageView* out) {
    if (!ctx || !out) return GKRT_ERR_INVALID_ARG;
    if (!ctx->d_output) return fail(ctx, GKRT_ERR_STATE, "gkrt_output_resize was not called");
    out->device_ptr = ctx->d_output;
    out->width = ctx->OW;
    out->height = ctx->OH;
    out->pitch_bytes = ctx->OW * 4;
    out->format = GKRT_FMT_BGRA8;
    return GKRT_OK;
}

int gkrt_copy_output_to_host(GkrtContext* ctx, void* dst, size_t dst_bytes, void* stream) {
    if (!ctx) return GKRT_ERR_INVALID_ARG;
    if (!ctx->d_output) return fail(ctx, GKRT_ERR_STATE, "gkrt_output_resize was not called");
    const size_t bytes = (size_t)ctx->OW * ctx->OH * 4;
    if (!dst || dst_bytes < bytes) return fail(ctx, GKRT_ERR_INVALID_ARG, "destination smaller than the image");
    DeviceGuard device_guard(ctx->device);
    GK_CUDA(cudaMemcpyAsync(dst, ctx->d_output, bytes, cudaMemcpyDeviceToHost, (cudaStream_t)stream));
    return gkrt_synchronize(ctx, stream);
}

int gkrt_screenshot(GkrtContext* ctx, uint32_t x, uint32_t y, uint32_t width, uint32_t height, void* dst,
                    size_t dst_bytes, void* stream) {
    if (!ctx) return GKRT_ERR_INVALID_ARG;
    if (!ctx->d_output) return fail(ctx, GKRT_ERR_STATE, "gkrt_output_resize was not called");
    if (width == 0 || height == 0 || (uint64_t)x + width > ctx->OW || (uint64_t)y + height > ctx->OH)
        return fail(ctx, GKRT_ERR_INVALID_ARG, "screenshot crop must lie inside the presentation image");
    const size_t bytes = (size_t)width * height * 3;
    if (!dst || dst_bytes < bytes) return fail(ctx, GKRT_ERR_INVALID_ARG, "destination smaller than the crop");
    DeviceGuard device_guard(ctx->device);
    const cudaStream_t st = (cudaStream_t)stream;
    uint8_t* d_rgb = nullptr;
    GK_CUDA(cudaMallocAsync((void**)&d_rgb, bytes, st));
    cudaError_t e = gkrt_launch_screenshot(ctx->d_output, (int)ctx->OW, (int)x, (int)y, (int)width, (int)height, d_rgb,
                                           st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dst, d_rgb, bytes, cudaMemcpyDeviceToHost, st);
    const cudaError_t ef = cudaFreeAsync(d_rgb, st);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "screenshot");
    if (ef != cudaSuccess) return cuda_fail(ctx, ef, "cudaFreeAsync(screenshot)");
    return gkrt_synchronize(ctx, stream);
}

int gkrt_upload_image(GkrtContext* ctx, int id, const void* src, size_t src_bytes, void* stream) {
    GkrtImageView v;
    int rc = gkrt_get_image(ctx, id, &v);
    if (rc != GKRT_OK) return rc;
    const size_t row = (size_t)v.width * image_bytes_per_px(id);
    if (!src || src_bytes != row * v.height) return fail(ctx, GKRT_ERR_INVALID_ARG, "source size differs from the image");
    DeviceGuard device_guard(ctx->device);
    GK_CUDA(cudaMemcpy2DAsync(v.device_ptr, v.pitch_bytes, src, row, row, v.height, cudaMemcpyHostToDevice,
                              (cudaStream_t)stream));
    return gkrt_synchronize(ctx, stream);
}

int gkrt_trace_rays(GkrtContext* ctx, const GkrtRay* rays, GkrtHit* hits, uint32_t count, uint32_t mode, void* stream) {
    if (!ctx) return GKRT_ERR_INVALID_ARG;
    if (count && (!rays || !hits)) return fail(ctx, GKRT_ERR_INVALID_ARG, "null ray or hit buffer");
    if (mode > GKRT_TRACE_ANY) return fail(ctx, GKRT_ERR_INVALID_ARG, "unknown trace mode");
    DeviceGuard device_guard(ctx->device);
    cudaStream_t st = (cudaStream_t)stream;
    int rc = ensure_bvh(ctx, 0, st);
    if (rc != GKRT_OK) return rc;
    GK_CUDA(cudaMemsetAsync(ctx->d_counters, 0, 6 * sizeof(unsigned long long), st));
    GK_CUDA(gkrt_launch_trace_rays(scene_view(ctx), rays, hits, count, mode, ctx->d_counters, st));
    return GKRT_OK;
}

// ---- ambient-cube probe grid ----

namespace {
constexpr size_t kProbeCount = (size_t)kProbeXY * kProbeXY * kProbeZ;
}

int gkrt_probe_voxelize(GkrtContext* ctx, void* stream) {
    if (!ctx) return GKRT_ERR_INVALID_ARG;
    if (!ctx->has_scene) return fail(ctx, GKRT_ERR_STATE, "no scene uploaded");
    DeviceGuard device_guard(ctx->device);
    cudaStream_t st = (cudaStream_t)stream;
    int rc = ensure_bvh(ctx, 0, st);
    if (rc != GKRT_OK) return rc;
    if (!ctx->d_cubes) GK_CUDA(cudaMalloc((void**)&ctx->d_cubes, kProbeCount * 14 * sizeof(uint32_t)));
    if (!ctx->d_voxels) GK_CUDA(cudaMalloc((void**)&ctx->d_voxels, kProbeCount * 4 * sizeof(uint32_t)));
    GK_CUDA(cudaMemsetAsync(ctx->d_cubes, 0, kProbeCount * 14 * sizeof(uint32_t), st));
    GK_CUDA(cudaMemsetAsync(ctx->d_counters, 0, 6 * sizeof(unsigned long long), st));
    GK_CUDA(gkrt_launch_probe_voxelize(shade_scene(ctx), 0, (uint32_t)kProbeCount, (uint4*)ctx->d_voxels,
                                       ctx->d_counters, st));
    return GKRT_OK;
}

int gkrt_probe_bake(GkrtContext* ctx, const GkrtFrameConstants* fc, uint32_t first, uint32_t count, void* stream) {
    if (!ctx || !fc) return GKRT_ERR_INVALID_ARG;
    if (!ctx->has_scene) return fail(ctx, GKRT_ERR_STATE, "no scene uploaded");
    if (!ctx->d_cubes || !ctx->d_voxels)
        return fail(ctx, GKRT_ERR_STATE, "no probe grid: upload one or call gkrt_probe_voxelize");
    if ((size_t)first + count > kProbeCount) return fail(ctx, GKRT_ERR_INVALID_ARG, "probe range outside the grid");
    if ((fc->flags & GKRT_FRAME_SKY_TEXTURE) && fc->sky_index >= GKRT_MAX_TEXTURES)
        return fail(ctx, GKRT_ERR_INVALID_ARG, "sky_index outside the texture pool");
    DeviceGuard device_guard(ctx->device);
    cudaStream_t st = (cudaStream_t)stream;
    int rc = ensure_bvh(ctx, 0, st);
    if (rc != GKRT_OK) return rc;
    if (!ctx->d_cubes_prev) GK_CUDA(cudaMalloc((void**)&ctx->d_cubes_prev, kProbeCount * 14 * sizeof(uint32_t)));
    GK_CUDA(cudaMemcpyAsync(ctx->d_cubes_prev, ctx->d_cubes, kProbeCount * 14 * sizeof(uint32_t),
                            cudaMemcpyDeviceToDevice, st));
    ProbeLight lt;
    std::memset(&lt, 0, sizeof(lt));
    if (!ctx->lights_host.empty()) {
        const GkrtLight& L = ctx->lights_host[0];
        if (L.light_mat_idx >= ctx->nmat) return fail(ctx, GKRT_ERR_INVALID_ARG, "light 0 has no material");
        // lerp(p1, p3, 0.5) as p1 + (p3 - p1) 0.5, one rounding per step
        lt.pos.x = std::fmaf(0.5f, L.p3[0] - L.p1[0], L.p1[0]);
        lt.pos.y = std::fmaf(0.5f, L.p3[1] - L.p1[1], L.p1[1]);
        lt.pos.z = std::fmaf(0.5f, L.p3[2] - L.p1[2], L.p1[2]);
        const float* dif = ctx->mat_host[L.light_mat_idx].diffuse;
        lt.power.x = dif[0]; lt.power.y = dif[1]; lt.power.z = dif[2]; lt.power.w = dif[3];
        lt.area = L.normal_area[3];
        lt.valid = 1;
    }
    GK_CUDA(cudaMemsetAsync(ctx->d_counters, 0, 6 * sizeof(unsigned long long), st));
    SkySH sh;
    std::memset(&sh, 0, sizeof(sh));
    if (fc->flags & GKRT_FRAME_SKY_TEXTURE) {
        sh.on = 1;
        if (!ctx->tex_sh.empty())
            std::memcpy(sh.c, ctx->tex_sh.data() + (size_t)fc->sky_index * 27u, sizeof(sh.c));
    }
    GK_CUDA(gkrt_launch_probe_bake(shade_scene(ctx), *fc, lt, sh, first, count, ctx->d_cubes_prev, ctx->d_cubes,
                                   (uint4*)ctx->d_voxels, ctx->d_counters, st));
    return GKRT_OK;
}

int gkrt_probe_download(GkrtContext* ctx, uint32_t* cubes, uint32_t* voxels) {
    if (!ctx) return GKRT_ERR_INVALID_ARG;
    if (!ctx->d_cubes || !ctx->d_voxels) return fail(ctx, GKRT_ERR_STATE, "no probe grid");
    DeviceGuard device_guard(ctx->device);
    GK_CUDA(cudaDeviceSynchronize());
    if (cubes) GK_CUDA(cudaMemcpy(cubes, ctx->d_cubes, kProbeCount * 14 * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    if (voxels) GK_CUDA(cudaMemcpy(voxels, ctx->d_voxels, kProbeCount * 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    return GKRT_OK;
}

int gkrt_get_stats(GkrtContext* ctx, GkrtStats* out) {
    if (!ctx || !out) return GKRT_ERR_INVALID_ARG;
    DeviceGuard device_guard(ctx->device);
    std::memset(out, 0, sizeof(*out));
    unsigned long long c[7] = {0, 0, 0, 0, 0, 0, 0};
    GK_CUDA(cudaDeviceSynchronize());
    GK_CUDA(cudaMemcpy(c, ctx->d_counters, sizeof(c), cudaMemcpyDeviceToHost));
    uint32_t errw = 0;
    GK_CUDA(cudaMemcpy(&errw, ctx->d_error, 4, cudaMemcpyDeviceToHost));
    out->rays_traced = c[0];
    out->exact_fallbacks = c[1];
    out->exact_retraces = c[2];
    out->node_visits = c[3];
    out->triangle_tests = c[4];
    out->rays_total = c[6];
    out->hit_fetches = c[5] > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)c[5];
    out->device_error = errw;
    out->bvh_nodes = ctx->blas_nodes_used;
    out->tlas_nodes = ctx->tlas_nodes;
    out->bvh_leaf_tris = ctx->nidx / 3;
    out->emitters = ctx->nemit;
    out->build_launches = gpu_bvh_launches(ctx->builder);
    out->wide_nodes = ctx->blas_wide_count + ctx->tlas_wide_count;
    out->wide_depth = (uint32_t)(ctx->blas_wide_depth + ctx->tlas_wide_depth);
    out->tlas_refits = ctx->tlas_refits;
    out->tlas_rebuilds = ctx->tlas_rebuilds;
    return GKRT_OK;
}

int gkrt_set_material_params(GkrtContext* ctx, const float* albedo_rgb, const float* roughness, uint32_t first,
                             uint32_t count, void* stream) {
    if (!ctx) return GKRT_ERR_INVALID_ARG;
    if (!ctx->has_scene) return fail(ctx, GKRT_ERR_STATE, "no scene uploaded");
    if ((uint64_t)first + count > ctx->nmat) return fail(ctx, GKRT_ERR_INVALID_ARG, "material range outside the scene");
    DeviceGuard device_guard(ctx->device);
    GK_CUDA(gkrt_launch_set_params(ctx->d_mat, albedo_rgb, roughness, first, count, (cudaStream_t)stream));
    return GKRT_OK;
}

// Error word of the context-free kernel entry points, one per device (allocated on first use,
// kept for the process).
static uint32_t* standalone_err_word() {
    static uint32_t* words[kMaxDevices] = {};
    const int dev = current_device_slot();
    if (dev < 0) return nullptr;
    if (!words[dev] && cudaMalloc((void**)&words[dev], 4) != cudaSuccess) return nullptr;
    return words[dev];
}

static int adjoint_checks(GkrtContext* ctx, const GkrtFrameConstants* fc, uint32_t spp) {
    int rc = check_frame(ctx, fc);
    if (rc != GKRT_OK) return rc;
    if (!ctx->has_scene) return fail(ctx, GKRT_ERR_STATE, "no scene uploaded");
    if (spp == 0 || spp > 4096) return fail(ctx, GKRT_ERR_INVALID_ARG, "spp must be 1..4096");
    if (fc->has_sun || fc->nee_mode != GKRT_NEE_REFERENCE)
        return fail(ctx, GKRT_ERR_UNSUPPORTED, "the adjoint covers the reference NEE mode without sun");
    if (fc->number_of_bounces > 16 || fc->max_number_of_bounces > 16)
        return fail(ctx, GKRT_ERR_UNSUPPORTED, "the adjoint records at most 16 bounces");
    if (ctx->nmat > 8192) return fail(ctx, GKRT_ERR_UNSUPPORTED, "the adjoint sums at most 8192 materials per block");
    if (ctx->textured || (fc->flags & GKRT_FRAME_SKY_TEXTURE))
        return fail(ctx, GKRT_ERR_UNSUPPORTED, "the adjoint covers untextured scenes under the constant sky");
    return GKRT_OK;
}

int gkrt_adjoint_forward(GkrtContext* ctx, const GkrtFrameConstants* fc, uint32_t spp, const float* sample_roughness,
                         float* image, void* stream) {
    int rc = adjoint_checks(ctx, fc, spp);
    if (rc != GKRT_OK) return rc;
    if (!image) return fail(ctx, GKRT_ERR_INVALID_ARG, "null image");
    DeviceGuard device_guard(ctx->device);
    cudaStream_t st = (cudaStream_t)stream;
    if ((rc = ensure_bvh(ctx, 0, st)) != GKRT_OK) return rc;
    GK_CUDA(cudaMemsetAsync(ctx->d_counters, 0, 6 * sizeof(unsigned long long), st));
    GK_CUDA(gkrt_launch_adjoint(shade_scene(ctx), *fc, (int)ctx->W, (int)ctx->H, spp, sample_roughness,
                                (float4*)image, nullptr, nullptr, nullptr, ctx->d_counters, st));
    return GKRT_OK;
}

int gkrt_adjoint_backward(GkrtContext* ctx, const GkrtFrameConstants* fc, uint32_t spp, const float* sample_roughness,
                          const float* d_image, double* grad_albedo, double* grad_roughness, void* stream) {
    int rc = adjoint_checks(ctx, fc, spp);
    if (rc != GKRT_OK) return rc;
    if (!d_image || !grad_albedo || !grad_roughness) return fail(ctx, GKRT_ERR_INVALID_ARG, "null buffer");
    DeviceGuard device_guard(ctx->device);
    cudaStream_t st = (cudaStream_t)stream;
    if ((rc = ensure_bvh(ctx, 0, st)) != GKRT_OK) return rc;
    GK_CUDA(cudaMemsetAsync(ctx->d_counters, 0, 6 * sizeof(unsigned long long), st));
    GK_CUDA(gkrt_launch_adjoint(shade_scene(ctx), *fc, (int)ctx->W, (int)ctx->H, spp, sample_roughness, nullptr,
                                (const float4*)d_image, grad_albedo, grad_roughness, ctx->d_counters, st));
    return GKRT_OK;
}

static int conv3x3_bf16(const void* x, uint32_t batch, uint32_t height, uint32_t width, uint32_t cin, const void* w,
                        const float* bias, uint32_t cout, void* y, uint32_t y_channels, uint32_t y_offset,
                        uint32_t y_store, uint32_t flags, void* pool, uint32_t pool_channels, uint32_t pool_offset,
                        void* up, uint32_t up_channels, uint32_t up_offset, void* stream) {
    if (!x || !w || !y || batch == 0 || height == 0 || width == 0 || batch > 65535 || height > 65535 ||
        width > 65535 || cin > 4096 || flags > 3u || pool_channels > 4096 || pool_offset > 4096 ||
        up_channels > 4096 || up_offset > 4096)
        return GKRT_ERR_INVALID_ARG;
    ConvArgs a{};
    a.B = (int)batch; a.H = (int)height; a.W = (int)width; a.cin = (int)cin; a.cout = (int)cout;
    a.x_c = (int)cin; a.x_off = 0;
    a.bias = bias;
    a.out = y;
    a.out_c = (int)y_channels;
    a.out_off = (int)y_offset;
    a.n_store = (int)y_store;
    a.flags = (int)flags;
    a.pool_out = pool; a.pool_c = (int)pool_channels; a.pool_off = (int)pool_offset;
    a.up_out = up; a.up_c = (int)up_channels; a.up_off = (int)up_offset;
    uint32_t* d_err = standalone_err_word();   // the standalone kernels' error word (this device's)
    if (!d_err) return GKRT_ERR_OOM;
    a.err = d_err;
    cudaError_t e = gkrt_launch_conv3x3(x, w, a, (cudaStream_t)stream);
    if (e == cudaErrorInvalidValue) return GKRT_ERR_INVALID_ARG;
    return e == cudaSuccess ? GKRT_OK : GKRT_ERR_CUDA;
}

int gkrt_conv3x3_bf16(const void* x, uint32_t batch, uint32_t height, uint32_t width, uint32_t cin, const void* w,
                      const float* bias, uint32_t cout, void* y, uint32_t y_channels, uint32_t y_offset,
                      uint32_t y_store, uint32_t flags, void* stream) {
    return conv3x3_bf16(x, batch, height, width, cin, w, bias, cout, y, y_channels, y_offset, y_store, flags, nullptr,
                        0, 0, nullptr, 0, 0, stream);
}

int gkrt_conv3x3_bf16_fused(const void* x, uint32_t batch, uint32_t height, uint32_t width, uint32_t cin,
                            const void* w, const float* bias, uint32_t cout, void* y, uint32_t y_channels,
                            uint32_t y_offset, uint32_t flags, void* pool, uint32_t pool_channels,
                            uint32_t pool_offset, void* up, uint32_t up_channels, uint32_t up_offset, void* stream) {
    if (flags & GKRT_CONV_F32) return GKRT_ERR_INVALID_ARG;
    return conv3x3_bf16(x, batch, height, width, cin, w, bias, cout, y, y_channels, y_offset, 0, flags, pool,
                        pool_channels, pool_offset, up, up_channels, up_offset, stream);
}

// ---- learned denoiser ----
// The caller holds a DeviceGuard for ctx->device.
static int unet_ready(GkrtContext* ctx) {
    if (!ctx->unet) return fail(ctx, GKRT_ERR_STATE, "gkrt_unet_init was not called");
    return GKRT_OK;
}
static int unet_size_ok(GkrtContext* ctx, uint32_t b, uint32_t h, uint32_t w) {
    if (b == 0 || b > 64 || h < 16 || w < 16 || h % 8 || w % 8 || h > 8192 || w > 8192)
        return fail(ctx, GKRT_ERR_INVALID_ARG, "batch 1..64, sizes multiples of 8 from 16 to 8192");
    return GKRT_OK;
}

int gkrt_unet_init(GkrtContext* ctx, uint64_t seed) {
    if (!ctx) return GKRT_ERR_INVALID_ARG;
    DeviceGuard device_guard(ctx->device);
    if (!ctx->unet && !(ctx->unet = gkrt_unet_new())) return fail(ctx, GKRT_ERR_OOM, "denoiser");
    GK_CUDA(gkrt_unet_init_params(ctx->unet, seed));
    return GKRT_OK;
}

int gkrt_unet_param_count(GkrtContext* ctx, uint32_t* count) {
    if (!ctx || !count) return GKRT_ERR_INVALID_ARG;
    DeviceGuard device_guard(ctx->device);
    if (!ctx->unet && !(ctx->unet = gkrt_unet_new())) return fail(ctx, GKRT_ERR_OOM, "denoiser");
    *count = (uint32_t)gkrt_unet_nparams(ctx->unet);
    return GKRT_OK;
}

int gkrt_unet_get_params(GkrtContext* ctx, float* params, float* grads) {
    if (!ctx) return GKRT_ERR_INVALID_ARG;
    DeviceGuard device_guard(ctx->device);
    int rc = unet_ready(ctx);
    if (rc != GKRT_OK) return rc;
    GK_CUDA(gkrt_unet_get_params_host(ctx->unet, params, grads));
    return GKRT_OK;
}

int gkrt_unet_get_state(GkrtContext* ctx, float* m, float* v, uint64_t* step) {
    if (!ctx) return GKRT_ERR_INVALID_ARG;
    DeviceGuard device_guard(ctx->device);
    int rc = unet_ready(ctx);
    if (rc != GKRT_OK) return rc;
    GK_CUDA(gkrt_unet_get_state_host(ctx->unet, m, v, step));
    return GKRT_OK;
}

int gkrt_unet_set_state(GkrtContext* ctx, const float* m, const float* v, uint64_t step) {
    if (!ctx) return GKRT_ERR_INVALID_ARG;
    DeviceGuard device_guard(ctx->device);
    int rc = unet_ready(ctx);
    if (rc != GKRT_OK) return rc;
    if (!m || !v || step > 0x7FFFFFFFull) return fail(ctx, GKRT_ERR_INVALID_ARG, "null moments or step out of range");
    GK_CUDA(gkrt_unet_set_state_host(ctx->unet, m, v, step));
    return GKRT_OK;
}

int gkrt_unet_set_params(GkrtContext* ctx, const float* params) {
    if (!ctx || !params) return GKRT_ERR_INVALID_ARG;
    DeviceGuard device_guard(ctx->device);
    if (!ctx->unet && !(ctx->unet = gkrt_unet_new())) return fail(ctx, GKRT_ERR_OOM, "denoiser");
    GK_CUDA(gkrt_unet_set_params_host(ctx->unet, params));
    return GKRT_OK;
}

int gkrt_unet_forward(GkrtContext* ctx, const float* input, uint32_t batch, uint32_t height, uint32_t width,
                      float* out_linear, float* out_raw, void* stream) {
    if (!ctx) return GKRT_ERR_INVALID_ARG;
    DeviceGuard device_guard(ctx->device);
    int rc = unet_ready(ctx);
    if (rc != GKRT_OK) return rc;
    if ((rc = unet_size_ok(ctx, batch, height, width)) != GKRT_OK) return rc;
    if (!input) return fail(ctx, GKRT_ERR_INVALID_ARG, "null input");
    GK_CUDA(gkrt_unet_forward_dev(ctx->unet, input, (int)batch, (int)height, (int)width, out_linear, out_raw,
                                  (cudaStream_t)stream));
    return GKRT_OK;
}

int gkrt_unet_backward(GkrtContext* ctx, const float* d_raw, void* stream) {
    if (!ctx) return GKRT_ERR_INVALID_ARG;
    DeviceGuard device_guard(ctx->device);
    int rc = unet_ready(ctx);
    if (rc != GKRT_OK) return rc;
    if (!d_raw) return fail(ctx, GKRT_ERR_INVALID_ARG, "null gradient");
    if (!gkrt_unet_has_forward(ctx->unet)) return fail(ctx, GKRT_ERR_STATE, "gkrt_unet_forward was not called");
    GK_CUDA(gkrt_unet_backward_dev(ctx->unet, d_raw, (cudaStream_t)stream));
    return GKRT_OK;
}

int gkrt_unet_zero_grad(GkrtContext* ctx, void* stream) {
    if (!ctx) return GKRT_ERR_INVALID_ARG;
    DeviceGuard device_guard(ctx->device);
    int rc = unet_ready(ctx);
    if (rc != GKRT_OK) return rc;
    GK_CUDA(gkrt_unet_zero_grad(ctx->unet, (cudaStream_t)stream));
    return GKRT_OK;
}

int gkrt_unet_train_step(GkrtContext* ctx, const float* input, const float* target, uint32_t batch, uint32_t height,
                         uint32_t width, float lr, double* loss, void* stream) {
    if (!ctx) return GKRT_ERR_INVALID_ARG;
    DeviceGuard device_guard(ctx->device);
    int rc = unet_ready(ctx);
    if (rc != GKRT_OK) return rc;
    if ((rc = unet_size_ok(ctx, batch, height, width)) != GKRT_OK) return rc;
    if (!input || !target || !(lr > 0.0f)) return fail(ctx, GKRT_ERR_INVALID_ARG, "null buffer or lr <= 0");
    GK_CUDA(gkrt_unet_train_step_dev(ctx->unet, input, target, (int)batch, (int)height, (int)width, lr, loss,
                                     (cudaStream_t)stream));
    return GKRT_OK;
}

int gkrt_conv3x3_wgrad_bf16(const void* dy, const void* x, uint32_t batch, uint32_t height, uint32_t width,
                            uint32_t cin, uint32_t cout, float* dw, void* stream) {
    if (!dy || !x || !dw || batch == 0 || height == 0 || width == 0 || batch > 65535 || height > 65535 ||
        width > 65535)
        return GKRT_ERR_INVALID_ARG;
    uint32_t* d_err = standalone_err_word();
    if (!d_err) return GKRT_ERR_OOM;
    WgradArgs a{};
    a.B = (int)batch; a.H = (int)height; a.W = (int)width;
    a.dp = (const __nv_bfloat16*)dy; a.dp_c = (int)cout; a.dp_off = 0; a.cout = (int)cout;
    a.x = (const __nv_bfloat16*)x; a.x_c = (int)cin; a.x_off = 0; a.cin = (int)cin;
    a.dw = dw;
    a.err = d_err;
    cudaError_t e = gkrt_launch_conv_wgrad(a, (cudaStream_t)stream);
    if (e == cudaErrorInvalidValue) return GKRT_ERR_INVALID_ARG;
    return e == cudaSuccess ? GKRT_OK : GKRT_ERR_CUDA;
}

int gkrt_affine_inverse(const float w[12], float winv[12]) {
    if (!w || !winv) return GKRT_ERR_INVALID_ARG;
    double a[3][3], t[3];
    for (int r = 0; r < 3; ++r) {
        for (int c = 0; c < 3; ++c) a[r][c] = w[4 * r + c];
        t[r] = w[4 * r + 3];
    }
    double det = a[0][0] * (a[1][1] * a[2][2] - a[1][2] * a[2][1]) - a[0][1] * (a[1][0] * a[2][2] - a[1][2] * a[2][0]) +
                 a[0][2] * (a[1][0] * a[2][1] - a[1][1] * a[2][0]);
    if (!(std::fabs(det) > 1e-30)) return GKRT_ERR_INVALID_ARG;
    double inv[3][3];
    inv[0][0] = (a[1][1] * a[2][2] - a[1][2] * a[2][1]) / det;
    inv[0][1] = (a[0][2] * a[2][1] - a[0][1] * a[2][2]) / det;
    inv[0][2] = (a[0][1] * a[1][2] - a[0][2] * a[1][1]) / det;
    inv[1][0] = (a[1][2] * a[2][0] - a[1][0] * a[2][2]) / det;
    inv[1][1] = (a[0][0] * a[2][2] - a[0][2] * a[2][0]) / det;
    inv[1][2] = (a[0][2] * a[1][0] - a[0][0] * a[1][2]) / det;
    inv[2][0] = (a[1][0] * a[2][1] - a[1][1] * a[2][0]) / det;
    inv[2][1] = (a[0][1] * a[2][0] - a[0][0] * a[2][1]) / det;
    inv[2][2] = (a[0][0] * a[1][1] - a[0][1] * a[1][0]) / det;
    for (int r = 0; r < 3; ++r) {
        double tt = 0.0;
        for (int c = 0; c < 3; ++c) {
            winv[4 * r + c] = (float)inv[r][c];
            tt -= inv[r][c] * t[c];
        }
        winv[4 * r + 3] = (float)tt;
    }
    return GKRT_OK;
}

}  // extern "C"
