// gkrt_internal.h — declarations shared by the host side of libgkrt and its kernels.
#pragma once
#include <cstdint>
#include <vector>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/gkrt.h"

namespace gk {
struct ShadeScene;
struct PixelImages;
struct SceneView;
struct BvhNode;
struct WideNode;
struct ProbeLight;
struct SkySH;

// Launch-geometry and attribute caches of the launchers are kept per device (a process may
// drive several GPUs): the current device's slot, or -1 past kMaxDevices.
constexpr int kMaxDevices = 64;
inline int current_device_slot() {
    int d = 0;
    if (cudaGetDevice(&d) != cudaSuccess || d < 0 || d >= kMaxDevices) return -1;
    return d;
}

// Makes `device` current for the life of the object and gives the caller's current device
// back at the end, so that an entry point leaves the calling thread's device as it found it.
// status: the cudaSetDevice result (entry points that report it check it).
struct DeviceGuard {
    int prev = -1;
    cudaError_t status = cudaSuccess;
    explicit DeviceGuard(int device) {
        if (cudaGetDevice(&prev) != cudaSuccess) {
            cudaGetLastError();
            prev = -1;
        }
        if (prev != device) status = cudaSetDevice(device);
    }
    ~DeviceGuard() {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
    DeviceGuard(const DeviceGuard&) = delete;
    DeviceGuard& operator=(const DeviceGuard&) = delete;
};

struct ReprojectArgs {
    int W, H, P;                   // P: row pitch in pixels (a multiple of 4)
    uint32_t progressive, temporal_frames;
    uint32_t* err;
    const float4 *src_d, *src_s, *src_a, *prev_d, *prev_s, *prev_a, *normal;
    const float2* motion;
    const uint32_t *id0, *id1, *moment;
    float4 *acc_d, *acc_s, *acc_a;
};

struct ComposeArgs {
    int W, H, P;
    uint32_t bf_size, hdr;
    float bf_sigma, bf_sigma_lum, paper_white_nit, pad;
    uint32_t* err;
    const float4 *acc_d, *acc_s, *acc_a;
    float4 *out, *out_linear;
};

struct AtrousArgs {
    int W, H, P;
    int step;                      // 1, 2, 4
    uint32_t last, hdr;            // last pass remodulates and tone maps
    float sigma_lum, paper_white_nit;
    uint32_t* err;
    const float4 *normal, *albedo, *spec;
    const uint32_t* id0;
    float4* out;                   // this pass's output (scratch)
    float4 *final_out, *final_linear;
};

// 3x3 convolution on the tensor cores (k_conv.cu). x: NHWC bf16 [B][H][W][cin];
// w: [cout][9][cin] bf16; out: NHWC with out_c channels, written at channel out_off.
constexpr int kConvRelu = 1, kConvF32Out = 2;
struct ConvArgs {
    int B, H, W, cin, cout;        // cin % 32 == 0; cout % 16 == 0, 16..256 (MMA N)
    int x_c, x_off;                // input: channel stride and first channel (multiple of 8)
    int x_valid;                   // channels the input holds at x_off (a multiple of 32 <= cin, or 16
                                   // for cin == 32 with Cout <= 32; 0: cin); the rest read as zeros
    const float* bias;             // cout floats or null
    void* out;
    int out_c, out_off;            // multiples of 16 (bf16 output)
    int n_store;                   // fp32 output: channels stored (<= cout)
    int flags;                     // kConvRelu | kConvF32Out
    uint32_t* err;                 // device error word
    // optional outputs of the bf16 epilogue (null: none), channel strides and offsets multiples
    // of 8: the 2 x 2 average of the stored values at half resolution (H / 2 x W / 2, blocks
    // wholly inside the image; the denoiser's 2 x 2 average pooling), and every stored value at
    // the four pixels of double resolution (2H x 2W; its nearest upsampling)
    void* pool_out;
    int pool_c, pool_off;
    void* up_out;
    int up_c, up_off;
    // optional addend of the bf16 epilogue (null: none), added to the sum before ReLU: at half
    // resolution (H / 2 x W / 2, H and W even), add_c channels per pixel (a multiple of 8, at
    // least 4 cout), output pixel (x, y) reading channels ((y & 1) 2 + (x & 1)) cout + c of
    // pixel (x / 2, y / 2): the four sub-pixel parities of a convolution over nearest-upsampled
    // input, computed at half resolution
    const void* add_par;
    int add_c;
};

// Host-side BVH build (binned SAH over boxes). Returns nodes in device layout and the leaf
// order of the primitives; refs follow the encoding of gk_trace.cuh.
struct HostBvh {
    std::vector<BvhNode> nodes;
    std::vector<uint32_t> order;
    int root = -1;
    int depth = 0;
};
// boxes: 6 floats per primitive (lo xyz, hi xyz). node_base: index of nodes[0] in the
// global node array; prim_base: global index of order[0] (leaf refs are global).
void build_bvh_host(const float* boxes, uint32_t n, uint32_t max_leaf, uint32_t node_base, uint32_t prim_base,
                    bool leaf_is_instance, HostBvh& out);

// Emissive-triangle table for GKRT_NEE_EMISSIVE (emitters.cu): 5 float4 per emitter and one
// alias entry (threshold, alias index bits) per emitter.
struct EmitterTable {
    std::vector<float4> geo;
    std::vector<float2> alias;
};
float emitter_luminance(const float* rgb);
// Triangles of each mesh grouped by the material slot of their vertex 0: out[16 * mesh + slot].
void mesh_slot_triangles(const GkrtMesh* meshes, uint32_t nmesh, const uint32_t* indices, const uint32_t* slots,
                         std::vector<std::vector<uint32_t>>& out);
void build_emitter_table(const GkrtInstance* inst, uint32_t ninst, const GkrtMesh* meshes, const float* pos,
                         const uint32_t* indices, const std::vector<std::vector<uint32_t>>& slot_tris,
                         const GkrtMaterial* mats, uint32_t nmat, EmitterTable& out);

// GPU builder (bvh_gpu.cu): same split rule and node layout, device scratch reused across
// builds. Results stay in the builder's memory until its next build.
struct GpuBvh;
struct GpuInstBox {                 // one instance for the instance-level build or refit
    float world[12];
    uint32_t mesh, inst, pad0, pad1;
};
struct GpuBvhResult {
    const BvhNode* nodes = nullptr; // node_count slots; refs already include node_base
    uint32_t node_count = 0;        // slots, including reserved ones left unused (zero)
    uint32_t nodes_used = 0;
    int depth = 0;
    const uint32_t* order = nullptr;   // leaf order of the primitives
    const float* root_box = nullptr;   // 6 per root
    std::vector<int> root_node;        // absolute node index per root, -1 for an empty root
};
GpuBvh* gpu_bvh_new();
void gpu_bvh_free(GpuBvh* b);
uint32_t gpu_bvh_launches(const GpuBvh* b);   // kernels launched by all its builds
// One tree per mesh over all meshes' triangles; writes the triangles in leaf order to
// tris_out (3 float4 per triangle).
cudaError_t gpu_bvh_build_meshes(GpuBvh* b, const float4* pos, const uint32_t* indices, const GkrtMesh* meshes,
                                 uint32_t nmesh, uint32_t node_base, float4* tris_out, GpuBvhResult* out,
                                 cudaStream_t st);
// The instance level in one cooperative launch and one host wait: a binned-SAH tree (the
// builder's rule, one instance per leaf) over the n records at `inst` (device; mesh_box: 6
// floats per mesh), root node_base, slots [node_base, node_base + node_count) of the device
// array `nodes` (node_cap >= n + 1 slots, zeroed first), collapsed into wide nodes
// [wide_base, wide_base + wide_count) of `wide` (wide_cap nodes in all), links recorded when
// non-null. res->error != 0: the build failed (non-finite transforms, more than 64 levels);
// the nodes are then unusable.
struct RefitLinks;
struct InstLevelResult {
    uint32_t node_count = 0, nodes_used = 0, wide_count = 0, error = 0;
    int depth = 0, wide_depth = 0;
};
// _launch enqueues the build on st; _finish waits for it (the one host wait) and returns its
// result. Host work in between overlaps the build.
cudaError_t gpu_bvh_build_instance_level_launch(GpuBvh* b, const GpuInstBox* inst, uint32_t n, const float* mesh_box,
                                               BvhNode* nodes, uint32_t node_base, uint32_t node_cap, WideNode* wide,
                                               uint32_t wide_base, uint32_t wide_cap, const RefitLinks* links,
                                               cudaStream_t st);
cudaError_t gpu_bvh_build_instance_level_finish(GpuBvh* b, InstLevelResult* res, cudaStream_t st);
bool gpu_bvh_cooperative_supported();   // the current device takes cooperative launches
// Collapse of two-child trees (device array bin, roots: node refs, -1 for none) into the
// compressed 8-wide nodes the kernels traverse, at out[wide_base ...) of an array of out_cap
// nodes. wroots: wide root per tree (-1 for none); count: wide nodes written; depth: levels.
// links: when non-null, the collapse also records what a refit of these trees needs.
struct RefitLinks;
cudaError_t gpu_bvh_collapse(GpuBvh* b, const BvhNode* bin, const std::vector<int>& roots, uint32_t wide_base,
                             WideNode* out, size_t out_cap, std::vector<int>& wroots, uint32_t* count, int* depth,
                             cudaStream_t st, const RefitLinks* links = nullptr);

// Links of the instance level for refits, recorded by its collapse. A slot is 2 * node + side:
// the half of two-child node `node` that holds one child's box and ref. Device arrays.
struct RefitLinks {
    int* parent = nullptr;     // per two-child node nbase + i: the slot holding its box; -1 at the root
    int* leaf = nullptr;       // per instance: the slot of its leaf; -1 when not in the tree
    int* wsrc = nullptr;       // 8 per wide node wbase + j: the slots of its children's boxes; -1 unused
    uint32_t nbase = 0, ncap = 0, ninst = 0, wbase = 0, wcap = 0;
};
// Refit of the instance level in place: the two-child boxes of the leaves from the instances'
// current transforms (inst: device, one record per instance index), unions up to the root, then
// the wide nodes [wbase, wbase + nw) re-quantized. arrive: ncap counters, zero between refits.
// Two launches, no host synchronisation; a wide node whose boxes cannot be quantized sets
// err_bit in *err (the traversal error word).
cudaError_t gpu_bvh_refit_instances(const RefitLinks& links, const GpuInstBox* inst, const float* mesh_box,
                                    BvhNode* nodes, float* ubox, uint32_t* arrive, WideNode* wide, uint32_t nw,
                                    uint32_t* err, uint32_t err_bit, cudaStream_t st);
}  // namespace gk

// Output stage (k_output.cu): src the tone-mapped image (W x H, pitch P pixels) into the
// presentation image out (OW x OH BGRA8 words). Resolve: linear blit onto the rectangle at
// (ox, oy) of ow x oh. FSR: the EASU compose with push constants offset and output size.
cudaError_t gkrt_launch_output_resolve(const float4* src, int W, int H, int P, uint32_t* out, int OW, int OH, int ox,
                                       int oy, int ow, int oh, cudaStream_t st);
cudaError_t gkrt_launch_output_fsr(const float4* src, int W, int H, int P, uint32_t* out, int OW, int OH, int offx,
                                   int offy, int outw, int outh, cudaStream_t st);
// rgb: w x h x 3 bytes of the crop at (x0, y0), which lies inside the OW-wide image
cudaError_t gkrt_launch_screenshot(const uint32_t* img, int OW, int x0, int y0, int w, int h, uint8_t* rgb,
                                   cudaStream_t st);

// stack_words: traversal stack entries per thread, at least the scene's two-child depth bound
// (mesh depth + instance depth + 3) and at most kStackSize. textured: the scene's materials
// name textures (the textured instantiation also runs when the frame samples a sky texture).
cudaError_t gkrt_launch_trace_pass(const gk::ShadeScene& sc, const GkrtFrameConstants& fc, int W, int H, int P,
                                   const gk::PixelImages& im, unsigned long long* counters, unsigned int* work,
                                   int num_sms, int stack_words, bool textured, cudaStream_t st);
// Probe grid (k_probes.cu): voxel distance data of probes [first, first + count), and one bake
// step of those probes reading neighbours from cubes_prev (a snapshot of cubes).
cudaError_t gkrt_launch_probe_voxelize(const gk::ShadeScene& sc, uint32_t first, uint32_t count, uint4* voxels,
                                       unsigned long long* counters, cudaStream_t st);
cudaError_t gkrt_launch_probe_bake(const gk::ShadeScene& sc, const GkrtFrameConstants& fc, const gk::ProbeLight& lt,
                                   const gk::SkySH& sh, uint32_t first, uint32_t count, const uint32_t* cubes_prev, uint32_t* cubes,
                                   uint4* voxels, unsigned long long* counters, cudaStream_t st);
cudaError_t gkrt_launch_trace_rays(const gk::SceneView& S, const GkrtRay* rays, GkrtHit* hits, uint32_t n,
                                   uint32_t mode, unsigned long long* counters, cudaStream_t st);
// Internal helpers for entry points defined outside gkrt_api.cu.
#include <string>
int gkrt_internal_fail(GkrtContext* ctx, int code, const std::string& msg);
// Scene view, statistics counters and device of a context whose scene and BVH are already
// built; GKRT_ERR_STATE otherwise (nothing is built or allocated here).
int gkrt_internal_ready_view(GkrtContext* ctx, gk::SceneView* view, unsigned long long** counters, int* device);

cudaError_t gkrt_launch_adjoint(const gk::ShadeScene& sc, const GkrtFrameConstants& fc, int W, int H, uint32_t spp,
                                const float* sample_rough, float4* image, const float4* dimage, double* g_alb,
                                double* g_rough, unsigned long long* counters, cudaStream_t st);
cudaError_t gkrt_launch_set_params(GkrtMaterial* mats, const float* alb, const float* rough, uint32_t first,
                                   uint32_t count, cudaStream_t st);
cudaError_t gkrt_launch_conv3x3(const void* x, const void* w, const gk::ConvArgs& args, cudaStream_t st);
// Weight gradient (k_unet.cu): dw[cout][9][cin] += sum_p dp[p][cout] * x[p + tap][cin].
namespace gk {
struct WgradArgs {
    int B, H, W;
    const __nv_bfloat16* dp;
    int dp_c, dp_off, cout;
    const __nv_bfloat16* x;
    int x_c, x_off, cin;
    int x_valid;                   // channels X holds at x_off (multiple of 8, <= cin; 0: cin), the rest zero
    float* dw;
    uint32_t* err;
};
}
cudaError_t gkrt_launch_conv_wgrad(const gk::WgradArgs& a, cudaStream_t st);
cudaError_t gkrt_launch_avgpool2_bwd(const void* dout, int dout_c, int dout_off, void* din, int din_c, int din_off,
                                     int B, int H, int W, int C, int accumulate, cudaStream_t st);
cudaError_t gkrt_launch_upsample2_bwd(const void* dout, int dout_c, int dout_off, void* din, int din_c, int din_off,
                                      int B, int h, int w, int C, cudaStream_t st);
cudaError_t gkrt_launch_relu_bwd(void* dy, int dy_c, int dy_off, const void* y, int y_c, int y_off, long long npix,
                                 int C, cudaStream_t st);
cudaError_t gkrt_launch_bias_grad(const void* dp, int dp_c, int dp_off, long long npix, int C, float* db,
                                  cudaStream_t st);
size_t gkrt_conv_smem_bytes(int cout);
// The learned denoiser (unet.cu).
namespace gk {
constexpr int kUnetLayers = 15;
constexpr float kUnetMaxLog = 12.0f;   // output log(1 + radiance) clamp before expm1
struct Unet;
}
gk::Unet* gkrt_unet_new();
void gkrt_unet_delete(gk::Unet* u);
size_t gkrt_unet_nparams(const gk::Unet* u);
cudaError_t gkrt_unet_init_params(gk::Unet* u, uint64_t seed);
cudaError_t gkrt_unet_set_params_host(gk::Unet* u, const float* h);
cudaError_t gkrt_unet_get_params_host(gk::Unet* u, float* params, float* grads);
cudaError_t gkrt_unet_get_state_host(gk::Unet* u, float* m, float* v, uint64_t* step);
cudaError_t gkrt_unet_set_state_host(gk::Unet* u, const float* m, const float* v, uint64_t step);
cudaError_t gkrt_unet_zero_grad(gk::Unet* u, cudaStream_t st);
cudaError_t gkrt_unet_forward_dev(gk::Unet* u, const float* input, int b, int h, int w, float* out_linear,
                                  float* out_raw, cudaStream_t st);
cudaError_t gkrt_unet_backward_dev(gk::Unet* u, const float* d_raw, cudaStream_t st);
bool gkrt_unet_has_forward(const gk::Unet* u);   // a forward ran (the backward's size and input)
cudaError_t gkrt_unet_train_step_dev(gk::Unet* u, const float* input, const float* target, int b, int h, int w,
                                     float lr, double* loss_host, cudaStream_t st);
cudaError_t gkrt_unet_denoise_frame(gk::Unet* u, const float4* sd, const float4* ss, const float4* alb,
                                    const float4* nrm, const float* depth, int W, int H, int P, float* y_out_raw,
                                    cudaStream_t st);
const float* gkrt_unet_output(const gk::Unet* u);
uint32_t* gkrt_unet_error_word(const gk::Unet* u);
// compose writer over the denoiser's log-space output (k_post.cu)
cudaError_t gkrt_launch_unet_compose(const gk::ComposeArgs& a, const float* y, cudaStream_t st);
cudaError_t gkrt_launch_reproject(const gk::ReprojectArgs& a, cudaStream_t st);
cudaError_t gkrt_launch_compose(const gk::ComposeArgs& a, cudaStream_t st);
cudaError_t gkrt_launch_atrous(const gk::AtrousArgs& a, const float4* in, float4* tmp0, float4* tmp1, cudaStream_t st);
