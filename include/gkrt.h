/*
 * gkrt.h — C ABI of the GB300-native ray-tracing pass.
 *
 * This is the drop-in boundary for gkNextRenderer's path-tracing logic renderer.
 * The reference plugs a "logic renderer" into its Vulkan frame loop
 * (class LogicRendererBase, src/Rendering/VulkanBaseRenderer.hpp:213-243), and the
 * path tracer implements it (src/Rendering/PathTracing/PathTracingRenderer.cpp:66-232).
 * Its inputs are the scene buffers addressed through the GPUScene push constant
 * (assets/shaders/common/BasicTypes.slang:261-291, filled by Scene::FetchGPUScene,
 * src/Assets/Scene.cpp:291-314) and the per-frame UniformBufferObject
 * (BasicTypes.slang:22-84, built by NextEngine::GetUniformBufferObject,
 * src/Runtime/Engine.cpp:736-849). Its outputs are bindless storage images
 * (assets/shaders/common/BindlessTexture.slang:8-40).
 *
 * Here the same pass is exposed as plain C: host pointers and sizes in, device images
 * out, every call returns a status code, no exceptions cross the boundary, and all GPU
 * work is ordered on the caller's CUDA stream (passed as void* so that this header
 * needs no CUDA include). One context is used by one host thread at a time.
 */
#ifndef GKRT_H
#define GKRT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GKRT_ABI_VERSION 2

/* ---- status codes (the reference throws instead: src/Utilities/Exception.hpp:10) ---- */
#define GKRT_OK                0
#define GKRT_ERR_INVALID_ARG   1  /* bad pointer, size, id, NaN vertex, ...            */
#define GKRT_ERR_OOM           2  /* device allocation failed                           */
#define GKRT_ERR_CUDA          3  /* a CUDA runtime call failed                         */
#define GKRT_ERR_TIMEOUT       4  /* a bounded wait ran out (host watchdog)             */
#define GKRT_ERR_DEVICE_LIMIT  5  /* a device loop hit its iteration cap                */
#define GKRT_ERR_UNSUPPORTED   6  /* feature outside this pass                           */
#define GKRT_ERR_STATE         7  /* call order: render before scene/resize, ...        */
#define GKRT_ERR_NO_DEVICE     8  /* no CUDA device / the kernels are not loadable      */

/* ---- material models (BasicTypes.slang:183-188) ---- */
#define GKRT_MAT_LAMBERTIAN    0u
#define GKRT_MAT_METALLIC      1u
#define GKRT_MAT_DIELECTRIC    2u
#define GKRT_MAT_ISOTROPIC     3u
#define GKRT_MAT_DIFFUSE_LIGHT 4u
#define GKRT_MAT_MIXTURE       5u

/* Material: byte-for-byte the reference's 64-byte Material (BasicTypes.slang:218-236).
 * Texture ids are -1 or ids of textures given to gkrt_texture_upload (below GKRT_MAX_TEXTURES). */
typedef struct GkrtMaterial {
    float    diffuse[4];
    int32_t  diffuse_texture_id;
    int32_t  mra_texture_id;
    int32_t  normal_texture_id;
    float    fuzziness;
    float    refraction_index;
    uint32_t material_model;
    float    metalness;
    float    refraction_index2;
    float    normal_texture_scale;
    float    reserved[3];
} GkrtMaterial;

/* Emissive quad: the reference's 80-byte LightObject (BasicTypes.slang:171-182). */
typedef struct GkrtLight {
    float    p0[4];
    float    p1[4];
    float    p3[4];
    float    normal_area[4];
    uint32_t light_mat_idx;
    uint32_t reserved[3];
} GkrtLight;

/* Mesh ranges: the first four words of the reference's ModelData (BasicTypes.slang:97-111).
 * index_offset/index_count address GkrtSceneDesc.indices; indices are relative to vertex_offset. */
typedef struct GkrtMesh {
    uint32_t index_offset;
    uint32_t index_count;
    uint32_t vertex_offset;
    uint32_t vertex_count;
} GkrtMesh;

/* Instance: the reference's NodeProxy (BasicTypes.slang:86-95) with affine 3x4 row-major
 * transforms instead of 4x4 ones, plus the world->object inverse that RayQuery derives
 * internally (CommittedRayWorldToObject, Shading.slang:808). Supplying the inverse keeps
 * the object-space ray identical for every consumer; gkrt_affine_inverse() computes it.
 * combined_prev maps this frame's world position to last frame's (Node::TickVelocity,
 * src/Assets/Node.cpp:82-106: prevTransform * inverse(transform)). */
typedef struct GkrtInstance {
    uint32_t instance_id;   /* custom index: written to the object-id image             */
    uint32_t mesh_id;       /* index into GkrtSceneDesc.meshes (NodeProxy.modelId)     */
    uint32_t visible;       /* 0: left out of the top-level BVH (instance mask 0)      */
    uint32_t reserved;
    float    world[12];
    float    world_inv[12];
    float    combined_prev[12];
    uint32_t mat_id[16];    /* per-vertex material slot -> material index              */
} GkrtInstance;

/* Scene: what Scene::RebuildMeshBuffer uploads (src/Assets/Scene.cpp:102-289) in FP32.
 * All arrays are host memory and are copied; the caller keeps ownership. */
typedef struct GkrtSceneDesc {
    const float*        positions;      /* float4 per vertex, w ignored                */
    const float*        normals;        /* float4 per vertex, w ignored                */
    const uint32_t*     material_slots; /* per vertex, 0..15 (packed in Vertex.hpp:97) */
    uint32_t            vertex_count;
    const uint32_t*     indices;
    uint32_t            index_count;
    const GkrtMesh*     meshes;
    uint32_t            mesh_count;
    const GkrtMaterial* materials;
    uint32_t            material_count;
    const GkrtInstance* instances;
    uint32_t            instance_count;
    const GkrtLight*    lights;
    uint32_t            light_count;
    /* Optional ambient-cube probe grid (AmbientCube.slang:12-15; 192*48*192 entries):
     * 14 u32 per AmbientCube and 4 u32 per VoxelData, or NULL for all-zero probes. */
    const uint32_t*     probe_cubes;
    const uint32_t*     probe_voxels;
    /* Optional vertex attributes of textured materials (GPUVertex, Vertex.hpp:80-99): the
     * texture coordinates (Position_Tx.w, Normal_Ty.w) and the object-space tangent with its
     * handedness in w. NULL: all zero. */
    const float*        texcoords;      /* float2 per vertex                               */
    const float*        tangents;       /* float4 per vertex                               */
} GkrtSceneDesc;

/* Frame constants: the fields of UniformBufferObject (BasicTypes.slang:22-84) the pass
 * reads, plus the reprojection push constants (PathTracingRenderer.cpp:127-128).
 * Matrices are column-major float[16] (glm's memory layout). */
typedef struct GkrtFrameConstants {
    float    model_view[16];
    float    projection[16];
    float    model_view_inverse[16];
    float    projection_inverse[16];
    float    view_projection[16];
    float    prev_view_projection[16];
    float    view_projection_unjit[16];
    float    prev_view_projection_unjit[16];
    float    sun_direction[4];
    float    sun_color[4];
    float    sky_color[4];          /* constant sky radiance (without GKRT_FRAME_SKY_TEXTURE) */
    float    aperture;
    float    focus_distance;
    float    paper_white_nit;
    float    sky_intensity;
    uint32_t total_frames;
    uint32_t number_of_samples;
    uint32_t number_of_bounces;
    uint32_t max_number_of_bounces;
    uint32_t temporal_frames;
    uint32_t has_sky;
    uint32_t has_sun;
    uint32_t taa;
    uint32_t fast_gather;
    uint32_t progressive_render;
    uint32_t bf_size;              /* 0: no bilateral filter                           */
    uint32_t hdr;
    float    bf_sigma;
    float    bf_sigma_lum;
    float    bf_sigma_normal;
    uint32_t denoiser;             /* GKRT_DENOISE_*                                    */
    uint32_t nee_mode;             /* GKRT_NEE_*                                        */
    uint32_t flags;                /* GKRT_FRAME_*                                      */
    uint32_t sky_index;            /* SkyIdx: texture of the HDR sky, with GKRT_FRAME_SKY_TEXTURE */
    float    sky_rotation;         /* SkyRotation (half turns)                          */
} GkrtFrameConstants;

#define GKRT_DENOISE_JBF     0u    /* reference single-pass joint bilateral filter      */
#define GKRT_DENOISE_ATROUS  1u    /* 5x5 edge-aware a-trous, 3 passes (no reference)   */
#define GKRT_DENOISE_UNET    2u    /* learned bf16 U-Net on the current 1-spp images    */

#define GKRT_NEE_REFERENCE   0u    /* sun-cone NEE only, as the built Slang path        */
#define GKRT_NEE_EMISSIVE    1u    /* + emissive-triangle NEE via an alias table (new)  */

#define GKRT_FRAME_PRIMARY_IDS  1u /* also write HIT_INST / HIT_PRIM of the camera ray  */
#define GKRT_FRAME_SKY_TEXTURE  2u /* sky misses sample texture sky_index as an equirect-
                                      angular map (SampleIBLV2, Shading.slang:194-199);
                                      without the flag the sky is sky_color              */

/* Textures (the reference's bindless GlobalTexturePool). Texels are stored as RGBA float:
 * RGBA8 UNORM decoded as c / 255, RGBA8 sRGB through the sRGB transfer function (alpha c / 255),
 * RGBA32F as given. Sampling follows the pool's sampler (Sampler.hpp:9-27, TextureImage.cpp:
 * 24-31) at level 0 (SampleLevel(uv, 0)): Vulkan's linear filter with repeat addressing. */
#define GKRT_TEX_RGBA8_UNORM 0u
#define GKRT_TEX_RGBA8_SRGB  1u
#define GKRT_TEX_RGBA32F     2u
#define GKRT_MAX_TEXTURES    4096u

/* Images owned by the context (formats: FP32x4 unless stated). */
#define GKRT_IMG_SINGLE_DIFFUSE    0
#define GKRT_IMG_SINGLE_SPECULAR   1
#define GKRT_IMG_ALBEDO            2
#define GKRT_IMG_NORMAL            3   /* xyz normal, w roughness                        */
#define GKRT_IMG_OBJECT_ID         4   /* u32, 65535 on a miss                           */
#define GKRT_IMG_OBJECT_ID_PREV    5   /* u32                                            */
#define GKRT_IMG_MOTION            6   /* FP32x2 pixel motion                            */
#define GKRT_IMG_PREV_DEPTH        7   /* FP32                                           */
#define GKRT_IMG_MOTION_MOMENT     8   /* u32                                            */
#define GKRT_IMG_ACCUM_DIFFUSE     9
#define GKRT_IMG_ACCUM_SPECULAR    10
#define GKRT_IMG_ACCUM_ALBEDO      11
#define GKRT_IMG_PREV_DIFFUSE      12
#define GKRT_IMG_PREV_SPECULAR     13
#define GKRT_IMG_PREV_ALBEDO       14
#define GKRT_IMG_DENOISED          15  /* tonemapped, as RT_DENOISED                     */
#define GKRT_IMG_DENOISED_LINEAR   16  /* same pixel before the tonemap                  */
#define GKRT_IMG_HIT_INST          17  /* u32 instance index of the camera-ray hit       */
#define GKRT_IMG_HIT_PRIM          18  /* u32 primitive index within the mesh            */
#define GKRT_IMG_COUNT             19

#define GKRT_FMT_F32X4  0
#define GKRT_FMT_F32X2  1
#define GKRT_FMT_F32    2
#define GKRT_FMT_U32    3

typedef struct GkrtImageView {
    void*    device_ptr;
    uint32_t width;
    uint32_t height;
    uint32_t pitch_bytes;
    uint32_t format;
} GkrtImageView;

/* Ray query records for gkrt_trace_rays (device memory). */
typedef struct GkrtRay {
    float origin[3];
    float tmin;
    float dir[3];
    float tmax;
} GkrtRay;

typedef struct GkrtHit {
    float    t;          /* hit distance; -1 on a miss                                  */
    float    b1, b2;     /* barycentrics of vertex 1 and 2                              */
    uint32_t inst;       /* instance index, 0xFFFFFFFF on a miss                        */
    uint32_t prim;       /* triangle index within the instance's mesh                   */
    uint32_t pad[3];
} GkrtHit;

#define GKRT_TRACE_CLOSEST 0u
#define GKRT_TRACE_ANY     1u

typedef struct GkrtDeviceDesc {
    int32_t  device;            /* CUDA ordinal                                          */
    uint32_t flags;             /* GKRT_DEVICE_*                                         */
    uint32_t watchdog_ms;       /* 0: default bounded wait for gkrt_synchronize          */
    uint32_t reserved;
} GkrtDeviceDesc;

/* Per-pass GPU timers, as the reference's SCOPED_GPU_TIMER scopes read back at frame end
 * (VulkanGpuTimer.hpp:12-120; scopes PathTracingRenderer.cpp:111,126,138,160 and "TLAS Update"
 * RayTraceBaseRenderer.cpp:209): with this flag each pass records an event pair on its stream.
 * Every pass also opens an NVTX range of the same name, with or without the flag. */
#define GKRT_DEVICE_PASS_TIMERS 1u
typedef struct GkrtPassTimes {  /* ms of each pass's last run, -1 if it has not run      */
    float rt_pass_ms;
    float reproject_pass_ms;
    float compose_pass_ms;       /* the denoise pass                                     */
    float copy_pass_ms;          /* gkrt_end_frame: a buffer swap, no GPU work           */
    float tlas_update_ms;        /* gkrt_scene_update_instances / _refit_instances        */
    float reserved[3];
} GkrtPassTimes;

typedef struct GkrtStats {
    uint64_t rays_traced;       /* camera + bounce + shadow rays of the last trace pass   */
    uint64_t exact_fallbacks;   /* triangle tests decided in FP64, last pass              */
    uint64_t exact_retraces;    /* t-ambiguous candidate pairs resolved in FP64           */
    uint64_t node_visits;       /* BVH nodes visited, last pass                           */
    uint64_t triangle_tests;    /* ray/triangle tests, last pass                          */
    uint64_t rays_total;        /* rays traced since the context was created              */
    uint32_t device_error;      /* device error word: 1 stack, 2 iteration cap, 4 TMA wait,
                                   8 a refit box the 8-wide nodes cannot quantize          */
    uint32_t bvh_nodes;
    uint32_t bvh_leaf_tris;
    uint32_t tlas_nodes;
    uint32_t emitters;          /* emissive triangles in the GKRT_NEE_EMISSIVE table      */
    uint32_t build_launches;    /* kernels launched by GPU BVH builds since creation      */
    uint32_t wide_nodes;        /* compressed 8-wide nodes traversed (mesh + instance)    */
    uint32_t wide_depth;        /* wide levels, deepest mesh tree + instance tree         */
    uint32_t tlas_refits;       /* instance-level refits since creation                   */
    uint32_t hit_fetches;       /* closest hits whose vertex, normal, material and instance
                                   data were read (hit reconstruction), last pass          */
    uint32_t tlas_rebuilds;     /* instance-level builds since creation (uploads included) */
    uint32_t pad;
} GkrtStats;

typedef struct GkrtContext GkrtContext;

/* Context lifetime (LogicRendererBase ctor/OnDeviceSet, VulkanBaseRenderer.hpp:216-219). */
int  gkrt_context_create(const GkrtDeviceDesc* desc, GkrtContext** out);
int  gkrt_context_destroy(GkrtContext* ctx);
const char* gkrt_last_error_message(const GkrtContext* ctx);
int  gkrt_abi_version(void);

/* Image set (CreateSwapChain/DeleteSwapChain, PathTracingRenderer.cpp:66-102;
 * formats of VulkanBaseRenderer::CreateRenderImages, VulkanBaseRenderer.cpp:429-463). */
int  gkrt_resize(GkrtContext* ctx, uint32_t width, uint32_t height);

/* Scene upload (Scene::RebuildMeshBuffer, Scene.cpp:102-289) and per-frame instance
 * update (Scene::UpdateNodesGpuDriven, Scene.cpp:443-492, with AfterUpdateScene,
 * RayTraceBaseRenderer.cpp:165-191). Instance updates keep mesh ids and count. */
int  gkrt_scene_upload(GkrtContext* ctx, const GkrtSceneDesc* scene);
int  gkrt_scene_update_instances(GkrtContext* ctx, const GkrtInstance* instances,
                                 uint32_t count, void* stream);
/* The same update with the instance level refit in place instead of rebuilt (the update mode
 * the reference's TLAS allows, VK_BUILD_ACCELERATION_STRUCTURE_ALLOW_UPDATE_BIT_KHR,
 * TopLevelAccelerationStructure.cpp:30): the tree keeps its topology, its boxes follow the new
 * transforms bottom-up and its 8-wide nodes are re-quantized, in two launches ordered on
 * `stream` with no host synchronisation. Trace results are identical to a rebuild's (the hit
 * rule does not depend on the tree); traversal cost grows as instances drift from the build's
 * layout, so callers rebuild now and then. When the set of instances in the tree changes
 * (visibility, or a mesh without triangles) it rebuilds instead. */
int  gkrt_scene_refit_instances(GkrtContext* ctx, const GkrtInstance* instances,
                                uint32_t count, void* stream);
/* The same update, refit or rebuild by the traversal cost the refits have cost so far: it refits
 * while the tree keeps its instances and the node visits per ray of the latest completed trace
 * pass are below growth_limit times those of the first completed pass after the last rebuild,
 * and rebuilds otherwise (then the next completed pass sets the new baseline). Each trace pass
 * copies its counters to page-locked memory without a host wait; the policy reads the newest
 * pass that has finished, so it may act one frame late. growth_limit >= 1 (1: rebuild every
 * time); gkrt_scene_update_instances and _refit_instances do not consult it. Counts of both
 * outcomes in GkrtStats (tlas_refits, tlas_rebuilds). */
int  gkrt_scene_update_instances_auto(GkrtContext* ctx, const GkrtInstance* instances, uint32_t count,
                                      float growth_limit, void* stream);

/* Acceleration structures (RayTraceBaseRenderer::CreateBottomLevelStructures /
 * CreateTopLevelStructures, RayTraceBaseRenderer.cpp:276-386; TLAS update :205-218).
 * flags: GKRT_BUILD_* */
#define GKRT_BUILD_BLAS 1u
#define GKRT_BUILD_TLAS 2u
#define GKRT_BUILD_ALL  3u
/* Build on the host CPU instead of the GPU builder. The choice sticks for later builds
 * (including the instance-level rebuild of gkrt_scene_update_instances) until a call
 * without the flag. Both builders use the same split rule; trace results are identical. */
#define GKRT_BUILD_ON_HOST 4u
int  gkrt_build_bvh(GkrtContext* ctx, uint32_t flags, void* stream);

/* Passes (PathTracingRenderer::Render, PathTracingRenderer.cpp:104-218). */
int  gkrt_trace_pass(GkrtContext* ctx, const GkrtFrameConstants* fc, void* stream);     /* "rt pass"        */
int  gkrt_reproject_pass(GkrtContext* ctx, const GkrtFrameConstants* fc, void* stream); /* "reproject pass" */
int  gkrt_denoise_pass(GkrtContext* ctx, const GkrtFrameConstants* fc, void* stream);   /* "compose pass"   */
int  gkrt_end_frame(GkrtContext* ctx, void* stream);                                    /* "copy pass"      */
/* All four in order: the whole Render() of the path-tracing logic renderer. */
int  gkrt_render_frame(GkrtContext* ctx, const GkrtFrameConstants* fc, void* stream);

/* Output stage: the presentation image, a headless device buffer of width x height 8-bit BGRA
 * words (byte order B, G, R, A) in place of the reference's B8G8R8A8_UNORM swapchain image
 * (SwapChain.cpp). Values convert as a UNORM store does: clamp to [0, 1] (NaN to 0), x 255,
 * round to nearest even. */
#define GKRT_FMT_BGRA8  4
#define GKRT_OUTPUT_RESOLVE 0   /* linear blit of the image onto the rectangle (offset, width x height):
                                   the resolve pass, VulkanBaseRenderer.cpp:1036-1068                 */
#define GKRT_OUTPUT_FSR     1   /* Process.UpScaleFSR.comp.slang: EASU from the render size to the
                                   presentation size when they differ, else a nearest copy; pixels
                                   [0, width/8*8) x [0, height/8*8) written at + offset; offset, width,
                                   height are its push constants (VulkanBaseRenderer.cpp:958-986)      */
typedef struct GkrtOutputDesc {
    uint32_t mode;              /* GKRT_OUTPUT_*                                              */
    int32_t  offset_x, offset_y;
    uint32_t width, height;
    uint32_t source_image;      /* image id read, normally GKRT_IMG_DENOISED                  */
} GkrtOutputDesc;
/* (Re)allocate the presentation image (SwapChain extent); contents start black (all zero).
 * width = height = 0 frees it. */
int  gkrt_output_resize(GkrtContext* ctx, uint32_t width, uint32_t height);
/* One output pass on `stream`; pixels outside the presentation image are not written. */
int  gkrt_output_pass(GkrtContext* ctx, const GkrtOutputDesc* desc, void* stream);
int  gkrt_get_output(GkrtContext* ctx, GkrtImageView* out);
/* The whole presentation image to host memory (width x height x 4 bytes); waits for `stream`. */
int  gkrt_copy_output_to_host(GkrtContext* ctx, void* dst, size_t dst_bytes, void* stream);
/* ScreenShot::SaveSwapChainToFileFast (ScreenShot.cpp:18-79): the crop (x, y, width, height) of
 * the presentation image as width x height x 3 bytes R, G, B, rows top to bottom, into dst (host
 * memory); waits for `stream`. The crop must lie inside the image. Encoding to a file is the
 * caller's (the Python layer writes PNG). */
int  gkrt_screenshot(GkrtContext* ctx, uint32_t x, uint32_t y, uint32_t width, uint32_t height,
                     void* dst, size_t dst_bytes, void* stream);

/* Waits for each pass's last recorded run and returns its GPU time (GKRT_ERR_STATE without
 * GKRT_DEVICE_PASS_TIMERS). */
int  gkrt_get_pass_times(GkrtContext* ctx, GkrtPassTimes* out);

/* Outputs (bindless storage images, BindlessTexture.slang:8-40). */
int  gkrt_get_image(GkrtContext* ctx, int image_id, GkrtImageView* out);
int  gkrt_copy_image_to_host(GkrtContext* ctx, int image_id, void* dst, size_t dst_bytes, void* stream);
/* The copy of gkrt_copy_image_to_host ordered on `stream` without waiting for it: the caller
 * synchronizes (the stream or an event recorded after the call) before reading dst, and keeps
 * the image unwritten until then. dst in page-locked memory makes the copy overlap later work
 * on other streams, as the reference's frames in flight overlap their readbacks
 * (VulkanBaseRenderer.cpp:727-869). */
int  gkrt_copy_image_to_host_async(GkrtContext* ctx, int image_id, void* dst, size_t dst_bytes, void* stream);
int  gkrt_upload_image(GkrtContext* ctx, int image_id, const void* src, size_t src_bytes, void* stream);

/* Texture `texture_id` (< GKRT_MAX_TEXTURES) of width x height texels (rows first to last, 4
 * channels in `format`, bytes = width * height * texel size), replacing an earlier texture of
 * that id. Materials name textures by id (diffuse, MRA, normal map); the sky by
 * GkrtFrameConstants.sky_index. An id without a texture samples as opaque white. An RGBA32F
 * texture is also projected on spherical harmonics for the probe bake's sky (ProjectHdrToSh,
 * Texture.cpp:180-254). Synchronous.
 * (GlobalTexturePool::CreateTextureImage / TextureImage, src/Assets/Texture.cpp:380-620.) */
int  gkrt_texture_upload(GkrtContext* ctx, uint32_t texture_id, uint32_t width, uint32_t height, uint32_t format,
                         const void* texels, size_t bytes);

/* Ray queries on the scene's BVH (FHardwareRayTracerV2::TraceRay / TraceOcclusion,
 * assets/shaders/common/Shading.slang:737-826). rays/hits are device pointers. A ray reports
 * hits with tmin <= t <= tmax (the reference's shaders pass TMin = EPS = 1e-3). Every entry
 * point of this header leaves the calling thread's current CUDA device as it found it. */
int  gkrt_trace_rays(GkrtContext* ctx, const GkrtRay* rays, GkrtHit* hits, uint32_t count,
                     uint32_t mode, void* stream);

/* The same ray queries for callers that cannot allocate device memory while they issue work
 * (a host engine whose device memory belongs to its own pool allocator, or a process at its
 * memory budget). No counterpart in the reference. The call allocates nothing: it needs a context
 * whose scene and BVH are already built (else GKRT_ERR_STATE), and its scratch memory is a
 * fixed 2 MiB static device array that every GPU loading the library keeps until process
 * exit. At most 4,194,304 rays per call (GKRT_ERR_INVALID_ARG above that). The first call on
 * a device looks up the array's device address; make that first call before any stream
 * capture. Calls share the array: calls that overlap on the GPU race, so order them on one
 * stream. Statistics land in the context's counters as for gkrt_trace_rays. */
int  gkrt_trace_rays_noalloc(GkrtContext* ctx, const GkrtRay* rays, GkrtHit* hits, uint32_t count,
                             uint32_t mode, void* stream);

/* Ambient-cube probe grid (AmbientCube.slang:12-15: 192 x 48 x 192 probes, 0.25 m apart from
 * (-24, -0.34375, -24); index y*192*192 + z*192 + x; 14 u32 per AmbientCube, 4 u32 per
 * VoxelData), read by the rt pass's path termination.
 *
 * gkrt_probe_voxelize: the distance data of every probe, computed on the GPU the way the
 * reference's CPU voxelizer computes it (VoxelizeCube, src/Assets/CPUAccelerationStructure.cpp:
 * 112-160: six axis rays of 16 m, diagonal rays in open space; a hit within 0.25 m on a back
 * face or an emitter marks the probe solid). Creates the grid when the scene had none, clears
 * the colours and resets the ages.
 *
 * gkrt_probe_bake: one bake step of probes [first, first + count) (the hw-lightbake dispatch
 * of RayTraceBaseRenderer::PostRender, RayTraceBaseRenderer.cpp:225-274, running
 * RenderAmbientCubeOnly, AmbientCube.slang:656-690): probes within 2 m of a surface trace 16
 * jittered rays per face, add sky, light 0 and sun, and blend into their colours with weight
 * 1/8. A ray that meets a surface takes its material's diffuse times its diffuse texture; a
 * sky miss takes, with GKRT_FRAME_SKY_TEXTURE, the spherical-harmonic projection of texture
 * sky_index (computed by gkrt_texture_upload for RGBA32F textures, zero for 8-bit ones:
 * SampleIBLRough, Shading.slang:188-192), else the constant sky colour. The reference's
 * schedule bakes slice (frame % F) of size (27648 / F) * 64 with F = 30, 120 or 300.
 * Neighbour probes are read as they were before the call.
 *
 * gkrt_probe_download: the grid to host memory (either pointer may be NULL); synchronous. */
int  gkrt_probe_voxelize(GkrtContext* ctx, void* stream);
int  gkrt_probe_bake(GkrtContext* ctx, const GkrtFrameConstants* fc, uint32_t first, uint32_t count, void* stream);
int  gkrt_probe_download(GkrtContext* ctx, uint32_t* cubes, uint32_t* voxels);

/* Differentiable rendering (no counterpart in the reference): the pass's estimator with
 * `spp` samples per pixel from the primary hit, composed as the compose pass composes it
 * (diffuse x primary albedo + specular, no filter), and its path-replay adjoint.
 * Reference NEE mode without sun, untextured materials and the constant sky (else
 * GKRT_ERR_UNSUPPORTED), at most 16 bounces.
 * image / d_image: dense width x height float4 device arrays (the context's size).
 * sample_roughness: per material, the roughness GGX directions are sampled with (detached);
 * NULL samples with the current roughness. GGX bounces are weighted by the ratio of the
 * sampler's densities at the current and the sampling roughness, which is 1 when they are
 * equal. Gradients are ADDED to grad_albedo (3 doubles per material) and grad_roughness
 * (1 double per material), device arrays the caller zeroes.
 * gkrt_set_material_params overwrites diffuse rgb (3 floats each) and fuzziness of
 * materials [first, first + count) from device arrays (either may be NULL); emitter
 * radiance changes need gkrt_scene_upload. */
int  gkrt_set_material_params(GkrtContext* ctx, const float* albedo_rgb, const float* roughness,
                              uint32_t first, uint32_t count, void* stream);
int  gkrt_adjoint_forward(GkrtContext* ctx, const GkrtFrameConstants* fc, uint32_t spp,
                          const float* sample_roughness, float* image, void* stream);
int  gkrt_adjoint_backward(GkrtContext* ctx, const GkrtFrameConstants* fc, uint32_t spp,
                           const float* sample_roughness, const float* d_image,
                           double* grad_albedo, double* grad_roughness, void* stream);

/* 3x3 "same" convolution on the tensor cores (building block of the learned denoiser; no
 * counterpart in the reference). x: NHWC bf16 [batch][height][width][cin], cin a multiple
 * of 32; w: bf16 [cout][3][3][cin], cout a multiple of 16 in 16..256; bias: cout floats or
 * NULL; y: NHWC with y_channels channels, written at channel y_offset (bf16, multiples of
 * 16), or fp32 with GKRT_CONV_F32 (then only y_store channels are written). Device
 * pointers, 16-byte aligned. */
/* Weight gradient of that convolution: dw[cout][3][3][cin] (fp32, ADDED to) = sum over pixels
 * of dy[p][cout] * x[p + tap][cin]; dy NHWC bf16 with cout channels (a multiple of 8, at most
 * 128), x with cin channels (a multiple of 16, at most 256). */
int  gkrt_conv3x3_wgrad_bf16(const void* dy, const void* x, uint32_t batch, uint32_t height, uint32_t width,
                             uint32_t cin, uint32_t cout, float* dw, void* stream);
#define GKRT_CONV_RELU 1u
#define GKRT_CONV_F32  2u
int  gkrt_conv3x3_bf16(const void* x, uint32_t batch, uint32_t height, uint32_t width, uint32_t cin,
                       const void* w, const float* bias, uint32_t cout, void* y, uint32_t y_channels,
                       uint32_t y_offset, uint32_t y_store, uint32_t flags, void* stream);
/* The same convolution (bf16 output) with the two extra outputs its epilogue can write, as the
 * denoiser's skip tensors use them (either pointer may be null): pool, NHWC bf16 at
 * (height / 2) x (width / 2) with pool_channels channels, at pool_offset the 2x2 average
 * (((0 + y00) + y01) + y10) + y11, times 1/4, of the stored bf16 outputs; up, NHWC bf16 at
 * (2 height) x (2 width) with up_channels channels, at up_offset each output repeated over its
 * 2x2 block (nearest upsampling). Channel counts and offsets multiples of 8. */
int  gkrt_conv3x3_bf16_fused(const void* x, uint32_t batch, uint32_t height, uint32_t width, uint32_t cin,
                             const void* w, const float* bias, uint32_t cout, void* y, uint32_t y_channels,
                             uint32_t y_offset, uint32_t flags, void* pool, uint32_t pool_channels,
                             uint32_t pool_offset, void* up, uint32_t up_channels, uint32_t up_offset, void* stream);

/* Learned denoiser (no counterpart in the reference, whose learned denoiser is the closed
 * OIDN library): a 4-level 3x3-convolution U-Net (32/64/96/128 channels) in bf16 with FP32
 * accumulation on the tensor cores, trained by this library's own forward and backward
 * kernels with Adam. input: dense float [batch][height][width][10] device array, channels
 * 1-spp linear radiance rgb, albedo rgb, normal xyz, NDC depth (clamped to [0, 1]); target:
 * [..][3] linear radiance.
 * out_linear: [..][4] denoised linear radiance (w = 1); out_raw: [..][4] the network's
 * log(1 + radiance) output in x, y, z (w: an unused fourth output), the quantity
 * gkrt_unet_backward's d_raw differentiates (its w is ignored). gkrt_unet_forward is the
 * inference forward: the first decoder convolution runs in its sub-pixel form at half
 * resolution (its taps over the upsampled input summed per output parity, the sums rounded to
 * bf16), within bf16 rounding of the training forward; gkrt_unet_backward re-runs the training
 * forward on the same input for the activations it needs (GKRT_ERR_STATE without a forward). Sizes
 * are multiples of 8 from 16 to 8192, batch 1..64. Parameters: gkrt_unet_param_count floats,
 * per layer the weights [cout][3][3][cin] then the biases; set_params resets Adam's state.
 * The denoise pass uses it with GKRT_DENOISE_UNET. */
int  gkrt_unet_init(GkrtContext* ctx, uint64_t seed);
int  gkrt_unet_param_count(GkrtContext* ctx, uint32_t* count);
int  gkrt_unet_get_params(GkrtContext* ctx, float* params, float* grads);
int  gkrt_unet_set_params(GkrtContext* ctx, const float* params);
/* Adam's first and second moments (gkrt_unet_param_count floats each, host memory) and its step
 * count, for checkpoints: restored after gkrt_unet_set_params, training resumes where it was. */
int  gkrt_unet_get_state(GkrtContext* ctx, float* m, float* v, uint64_t* step);
int  gkrt_unet_set_state(GkrtContext* ctx, const float* m, const float* v, uint64_t step);
int  gkrt_unet_forward(GkrtContext* ctx, const float* input, uint32_t batch, uint32_t height, uint32_t width,
                       float* out_linear, float* out_raw, void* stream);
int  gkrt_unet_backward(GkrtContext* ctx, const float* d_raw, void* stream);
int  gkrt_unet_zero_grad(GkrtContext* ctx, void* stream);
int  gkrt_unet_train_step(GkrtContext* ctx, const float* input, const float* target, uint32_t batch,
                          uint32_t height, uint32_t width, float lr, double* loss, void* stream);

int  gkrt_get_stats(GkrtContext* ctx, GkrtStats* out);
int  gkrt_synchronize(GkrtContext* ctx, void* stream);

/* Helper: world->object inverse of an affine 3x4 row-major transform, in FP64. */
int  gkrt_affine_inverse(const float world[12], float world_inv[12]);

#ifdef __cplusplus
}
#endif

#endif /* GKRT_H */
