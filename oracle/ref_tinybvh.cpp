// ref_tinybvh.cpp — a C shim over the reference's own CPU BVH library (test infrastructure).
//
// gkNextEngine vendors tinybvh v1.3.8 (src/ThirdParty/tinybvh/tiny_bvh.h) and uses it for
// its CPU ray casts (src/Assets/CPUAccelerationStructure.cpp:44-66, 172-313). This file is
// compiled against that header where it lies in the reference tree (oracle.build_ref());
// the header itself is not part of this repository. The shim exposes:
//   * closest hits of rays on a triangle soup with BVH_Double (double-precision
//     Moller-Trumbore, tiny_bvh.h:6487-6547) — used to pin the oracle's FP64 closest hit;
//   * closest hits with the single-precision BVH (tiny_bvh.h:2245-2292) over OpenMP
//     threads — the reference's own CPU traversal, timed as a CPU baseline.
#define TINYBVH_IMPLEMENTATION
#include "tiny_bvh.h"

#include <cstdint>
#include <cstring>
#include <vector>

extern "C" {

// verts: 9 doubles per triangle. rays: 6 doubles (origin, direction). Outputs t (hit.t;
// the library normalises the direction, so t is the distance) and prim (-1 on a miss).
void gkref_closest_double(const double* verts, int64_t ntri, const double* rays, int64_t nray, double* t_out,
                          int64_t* prim_out) {
    std::vector<tinybvh::bvhdbl3> v((size_t)ntri * 3);
    for (int64_t i = 0; i < ntri * 3; ++i) v[i] = tinybvh::bvhdbl3(verts[3 * i], verts[3 * i + 1], verts[3 * i + 2]);
    tinybvh::BVH_Double bvh;
    bvh.Build(v.data(), (uint64_t)ntri);
    for (int64_t r = 0; r < nray; ++r) {
        const double* q = rays + 6 * r;
        tinybvh::RayEx ray(tinybvh::bvhdbl3(q[0], q[1], q[2]), tinybvh::bvhdbl3(q[3], q[4], q[5]));
        bvh.Intersect(ray);
        if (ray.hit.t < BVH_DBL_FAR) {
            t_out[r] = ray.hit.t;
            prim_out[r] = (int64_t)ray.hit.prim;
        } else {
            t_out[r] = -1.0;
            prim_out[r] = -1;
        }
    }
}

// Single-precision traversal timing: returns hits found; threads via OpenMP.
int64_t gkref_closest_float(const float* verts4, int64_t ntri, const float* rays, int64_t nray, float* t_out,
                            int32_t* prim_out) {
    tinybvh::BVH bvh;
    bvh.Build((const tinybvh::bvhvec4*)verts4, (uint32_t)ntri);
    int64_t hits = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : hits)
    for (int64_t r = 0; r < nray; ++r) {
        const float* q = rays + 6 * r;
        tinybvh::Ray ray(tinybvh::bvhvec3(q[0], q[1], q[2]), tinybvh::bvhvec3(q[3], q[4], q[5]));
        bvh.Intersect(ray);
        bool h = ray.hit.t < BVH_FAR;
        t_out[r] = h ? ray.hit.t : -1.0f;
        prim_out[r] = h ? (int32_t)ray.hit.prim : -1;
        hits += h ? 1 : 0;
    }
    return hits;
}

}  // extern "C"
