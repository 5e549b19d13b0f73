/* A C (not C++) client of libgkrt through include/gkrt.h only: the boundary the reference's
 * renderer would call. Mode "cpu": the ABI version, host-only helpers and argument errors (no
 * CUDA work). Mode "gpu": a context, a one-quad scene, one rt pass of 16 x 16 pixels with
 * camera-ray ids, the ids read back to host memory, and the error path of a bad image id.
 * Prints "ok" and exits 0 on success. */
#include <math.h>
#include <stdio.h>
#include <string.h>

#include "gkrt.h"

static int fails = 0;
#define CHECK(c)                                                   \
    do {                                                           \
        if (!(c)) {                                                \
            fprintf(stderr, "check failed: %s (line %d)\n", #c, __LINE__); \
            ++fails;                                               \
        }                                                          \
    } while (0)

static void ident16(float* m) {
    memset(m, 0, 16 * sizeof(float));
    m[0] = m[5] = m[10] = m[15] = 1.0f;
}

static int cpu_checks(void) {
    CHECK(gkrt_abi_version() == GKRT_ABI_VERSION);
    /* host-only helper: inverse of a scaled, translated transform */
    const float w[12] = {2, 0, 0, 1, 0, 4, 0, 2, 0, 0, 8, 3};
    float wi[12];
    CHECK(gkrt_affine_inverse(w, wi) == GKRT_OK);
    CHECK(fabsf(wi[0] - 0.5f) < 1e-6f && fabsf(wi[3] + 0.5f) < 1e-6f && fabsf(wi[11] + 0.375f) < 1e-6f);
    /* argument errors are status codes, never crashes */
    CHECK(gkrt_context_create(NULL, NULL) == GKRT_ERR_INVALID_ARG);
    CHECK(gkrt_context_destroy(NULL) == GKRT_ERR_INVALID_ARG);
    CHECK(gkrt_resize(NULL, 16, 16) == GKRT_ERR_INVALID_ARG);
    CHECK(gkrt_last_error_message(NULL) != NULL);
    return fails;
}

static int gpu_checks(void) {
    GkrtDeviceDesc d = {0, 0, 5000, 0};
    GkrtContext* ctx = NULL;
    CHECK(gkrt_context_create(&d, &ctx) == GKRT_OK && ctx);
    if (!ctx) return fails;
    CHECK(gkrt_resize(ctx, 16, 16) == GKRT_OK);
    /* one quad at z = 5 facing the camera, spanning x, y in [-10, 10] */
    const float pos[16] = {-10, -10, 5, 1, 10, -10, 5, 1, 10, 10, 5, 1, -10, 10, 5, 1};
    const float nrm[16] = {0, 0, -1, 0, 0, 0, -1, 0, 0, 0, -1, 0, 0, 0, -1, 0};
    const uint32_t slots[4] = {0, 0, 0, 0};
    const uint32_t idx[6] = {0, 1, 2, 0, 2, 3};
    GkrtMesh mesh = {0, 6, 0, 4};
    GkrtMaterial mat;
    memset(&mat, 0, sizeof(mat));
    mat.diffuse[0] = mat.diffuse[1] = mat.diffuse[2] = 0.5f;
    mat.diffuse[3] = 1.0f;
    mat.diffuse_texture_id = mat.mra_texture_id = mat.normal_texture_id = -1;
    mat.fuzziness = 1.0f;
    mat.refraction_index = 1.0f;
    GkrtInstance inst;
    memset(&inst, 0, sizeof(inst));
    inst.instance_id = 7;
    inst.visible = 1;
    const float id12[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
    memcpy(inst.world, id12, sizeof(id12));
    memcpy(inst.world_inv, id12, sizeof(id12));
    memcpy(inst.combined_prev, id12, sizeof(id12));
    GkrtSceneDesc sd;
    memset(&sd, 0, sizeof(sd));
    sd.positions = pos; sd.normals = nrm; sd.material_slots = slots; sd.vertex_count = 4;
    sd.indices = idx; sd.index_count = 6; sd.meshes = &mesh; sd.mesh_count = 1;
    sd.materials = &mat; sd.material_count = 1; sd.instances = &inst; sd.instance_count = 1;
    CHECK(gkrt_scene_upload(ctx, &sd) == GKRT_OK);
    /* identity camera at the origin looking down +z; 1 spp, 1 bounce, ids of the camera ray */
    GkrtFrameConstants fc;
    memset(&fc, 0, sizeof(fc));
    ident16(fc.model_view); ident16(fc.projection); ident16(fc.model_view_inverse);
    ident16(fc.projection_inverse); ident16(fc.view_projection); ident16(fc.prev_view_projection);
    ident16(fc.view_projection_unjit); ident16(fc.prev_view_projection_unjit);
    fc.focus_distance = 1.0f;
    fc.paper_white_nit = 600.0f;
    fc.number_of_samples = 1; fc.number_of_bounces = 1; fc.max_number_of_bounces = 1;
    fc.temporal_frames = 1;
    fc.flags = GKRT_FRAME_PRIMARY_IDS;
    CHECK(gkrt_trace_pass(ctx, &fc, NULL) == GKRT_OK);
    uint32_t ids[256], prims[256], obj[256];
    CHECK(gkrt_copy_image_to_host(ctx, GKRT_IMG_HIT_INST, ids, sizeof(ids), NULL) == GKRT_OK);
    CHECK(gkrt_copy_image_to_host(ctx, GKRT_IMG_HIT_PRIM, prims, sizeof(prims), NULL) == GKRT_OK);
    CHECK(gkrt_copy_image_to_host(ctx, GKRT_IMG_OBJECT_ID, obj, sizeof(obj), NULL) == GKRT_OK);
    int hits = 0;
    for (int i = 0; i < 256; ++i) hits += (ids[i] == 0u && prims[i] < 2u && obj[i] == 7u);
    CHECK(hits == 256);
    GkrtStats st;
    CHECK(gkrt_get_stats(ctx, &st) == GKRT_OK && st.rays_traced >= 256 && st.device_error == 0);
    /* errors stay status codes on a live context */
    CHECK(gkrt_copy_image_to_host(ctx, 99, ids, sizeof(ids), NULL) == GKRT_ERR_INVALID_ARG);
    CHECK(strlen(gkrt_last_error_message(ctx)) > 0);
    CHECK(gkrt_context_destroy(ctx) == GKRT_OK);
    return fails;
}

int main(int argc, char** argv) {
    const int gpu = argc > 1 && strcmp(argv[1], "gpu") == 0;
    cpu_checks();
    if (gpu) gpu_checks();
    if (fails) return 1;
    printf("ok\n");
    return 0;
}
