// Ray queries against the device BVH: the two RT callbacks of the reference backends,
// RT::intersect (closest hit; libhussar/src/arch/cpu.cpp:63-87,
// src/arch/gpu/device/kernel.cu:45-63,76-98) and RT::visible (any hit / occlusion;
// cpu.cpp:53-61, kernel.cu:24-43,105-107).
//
// Triangle test: Moller-Trumbore in FP32 with the same operation order as the CPU
// restatement; a hit needs tnear < t <= tfar; equal-t ties go to the lower original
// primitive id, so the answer does not depend on the BVH shape or traversal order.
// Box test: slab test with fused multiply-adds on boxes padded at build time (the
// padding absorbs the rounding); 1/d is kept finite (see safe_inv).
#pragma once
#include "hsr_common.cuh"

namespace hsr {

constexpr int kTraversalStack = 64;

struct RayPre {
    float ox, oy, oz;
    float ix, iy, iz;      // 1 / d
    float oix, oiy, oiz;   // o / d products for the FMA slab test
};

// Direction components below 1e-30 in magnitude are replaced by +-1e-30 before the
// division, so 1/d stays finite: an exact zero would make the FMA slab form evaluate
// inf - inf = NaN on one plane and reject a box the (axis-parallel) ray lies in. The
// planes' distances are then about +-|x - o| * 1e30, far below FLT_MAX for any scene
// coordinate, and the FMA cancellation error (~6e-8 |o|) stays below the boxes' padding.
__device__ __forceinline__ float safe_inv(float d) {
    return 1.f / (fabsf(d) >= 1e-30f ? d : copysignf(1e-30f, d));
}

__device__ __forceinline__ RayPre ray_pre(f3 o, f3 d) {
    RayPre r;
    r.ox = o.x;
    r.oy = o.y;
    r.oz = o.z;
    r.ix = safe_inv(d.x);
    r.iy = safe_inv(d.y);
    r.iz = safe_inv(d.z);
    r.oix = o.x * r.ix;
    r.oiy = o.y * r.iy;
    r.oiz = o.z * r.iz;
    return r;
}

// Both child boxes of a node at once. Returns bit0/bit1 for child hits and the entry distances.
__device__ __forceinline__ int box2(const DNode &n, const RayPre &r, float tnear, float tfar, float &t0, float &t1) {
    float a0x = __fmaf_rn(n.a.x, r.ix, -r.oix), a1x = __fmaf_rn(n.a.y, r.ix, -r.oix);
    float a0y = __fmaf_rn(n.a.z, r.iy, -r.oiy), a1y = __fmaf_rn(n.a.w, r.iy, -r.oiy);
    float a0z = __fmaf_rn(n.c.x, r.iz, -r.oiz), a1z = __fmaf_rn(n.c.y, r.iz, -r.oiz);
    float b0x = __fmaf_rn(n.b.x, r.ix, -r.oix), b1x = __fmaf_rn(n.b.y, r.ix, -r.oix);
    float b0y = __fmaf_rn(n.b.z, r.iy, -r.oiy), b1y = __fmaf_rn(n.b.w, r.iy, -r.oiy);
    float b0z = __fmaf_rn(n.c.z, r.iz, -r.oiz), b1z = __fmaf_rn(n.c.w, r.iz, -r.oiz);
    float tmin0 = fmaxf(fmaxf(fminf(a0x, a1x), fminf(a0y, a1y)), fmaxf(fminf(a0z, a1z), tnear));
    float tmax0 = fminf(fminf(fmaxf(a0x, a1x), fmaxf(a0y, a1y)), fminf(fmaxf(a0z, a1z), tfar));
    float tmin1 = fmaxf(fmaxf(fminf(b0x, b1x), fminf(b0y, b1y)), fmaxf(fminf(b0z, b1z), tnear));
    float tmax1 = fminf(fminf(fmaxf(b0x, b1x), fmaxf(b0y, b1y)), fminf(fmaxf(b0z, b1z), tfar));
    t0 = tmin0;
    t1 = tmin1;
    int m = 0;
    if (tmin0 <= tmax0 * 1.0000004f) m |= 1;
    if (tmin1 <= tmax1 * 1.0000004f) m |= 2;
    return m;
}

// A node is two 32-byte sectors. On the device each is fetched by one 256-bit
// read-only load (nodes are 64-byte aligned), so a warp's node fetch costs the L1 two
// sector accesses per lane instead of four with 16-byte loads: traversal of dense scenes
// is bound by L1 throughput, not by L2 or DRAM.
__device__ __forceinline__ DNode load_node(const DNode *__restrict__ nodes, int i) {
    DNode n;
#ifdef __CUDA_ARCH__
    const float *p = reinterpret_cast<const float *>(nodes + i);
    int dx, dy, dz, dw;
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(n.a.x), "=f"(n.a.y), "=f"(n.a.z), "=f"(n.a.w), "=f"(n.b.x), "=f"(n.b.y), "=f"(n.b.z), "=f"(n.b.w)
        : "l"(p));
    asm("ld.global.nc.v8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(n.c.x), "=f"(n.c.y), "=f"(n.c.z), "=f"(n.c.w), "=r"(dx), "=r"(dy), "=r"(dz), "=r"(dw)
        : "l"(p + 8));
    n.d = make_int4(dx, dy, dz, dw);
#else
    const float4 *p = reinterpret_cast<const float4 *>(nodes + i);
    n.a = __ldg(p + 0);
    n.b = __ldg(p + 1);
    n.c = __ldg(p + 2);
    float4 d = __ldg(p + 3);
    n.d = make_int4(__float_as_int(d.x), __float_as_int(d.y), __float_as_int(d.z), __float_as_int(d.w));
#endif
    return n;
}

// Moller-Trumbore (same expression order as the CPU restatement). Returns t or -1.
__device__ __forceinline__ bool tri_test(const DTri &T, f3 o, f3 d, float tnear, float tfar, float &t_out) {
    f3 v0 = mk3(T.v0.x, T.v0.y, T.v0.z);
    f3 e1 = mk3(T.e1.x, T.e1.y, T.e1.z);
    f3 e2 = mk3(T.e2.x, T.e2.y, T.e2.z);
    f3 pv = crs3(d, e2);
    float det = dot3(e1, pv);
    if (det == 0.f) return false;
    float inv = 1.f / det;
    f3 tv = sub3(o, v0);
    float u = dot3(tv, pv) * inv;
    if (u < 0.f || u > 1.f) return false;
    f3 qv = crs3(tv, e1);
    float v = dot3(d, qv) * inv;
    if (v < 0.f || u + v > 1.f) return false;
    float t = dot3(e2, qv) * inv;
    if (!(t > tnear && t <= tfar)) return false;
    t_out = t;
    return true;
}

__device__ __forceinline__ DTri load_tri(const DTri *__restrict__ tris, int i) {
    const float4 *p = reinterpret_cast<const float4 *>(tris + i);
    DTri t;
    t.v0 = __ldg(p + 0);
    t.e1 = __ldg(p + 1);
    t.e2 = __ldg(p + 2);
    return t;
}

struct TraversalCounters {
    unsigned nodes;
    unsigned tris;
};

// Closest hit. Returns the triangle slot (or -1); t_best holds its distance.
template <bool kCount>
__device__ __forceinline__ int closest_hit(const DNode *__restrict__ nodes, const DTri *__restrict__ tris, f3 o, f3 d,
                                           float tnear, float tfar, float &t_best, int &prim_best,
                                           unsigned *status, TraversalCounters *cnt) {
    RayPre rp = ray_pre(o, d);
    int stack[kTraversalStack];
    int sp = 0;
    int node = 0;
    int best = -1;
    prim_best = 0x7fffffff;
    t_best = tfar;
    while (true) {
        if (node >= 0) {
            DNode n = load_node(nodes, node);
            if (kCount) cnt->nodes++;
            float t0, t1;
            int m = box2(n, rp, tnear, t_best, t0, t1);
            if (m == 3) {
                int nearC = n.d.x, farC = n.d.y;
                if (t1 < t0) {
                    nearC = n.d.y;
                    farC = n.d.x;
                }
                if (sp < kTraversalStack) {
                    stack[sp++] = farC;
                } else {
                    atomicOr(status, kStatusStackOverflow);
                }
                node = nearC;
                continue;
            } else if (m == 1) {
                node = n.d.x;
                continue;
            } else if (m == 2) {
                node = n.d.y;
                continue;
            }
        } else {
            const int ref = ~node;
            const int last = (ref >> 3) + (ref & 7);
            for (int slot = ref >> 3; slot <= last; ++slot) {
                DTri T = load_tri(tris, slot);
                if (kCount) cnt->tris++;
                float t;
                if (tri_test(T, o, d, tnear, tfar, t)) {
                    int prim = __float_as_int(T.v0.w);
                    if (t < t_best || (t == t_best && prim < prim_best)) {
                        t_best = t;
                        prim_best = prim;
                        best = slot;
                    }
                }
            }
        }
        if (sp == 0) break;
        node = stack[--sp];
    }
    return best;
}

// Any hit in (tnear, tfar]: true if occluded.
template <bool kCount>
__device__ __forceinline__ bool any_hit(const DNode *__restrict__ nodes, const DTri *__restrict__ tris, f3 o, f3 d,
                                        float tnear, float tfar, unsigned *status, TraversalCounters *cnt) {
    RayPre rp = ray_pre(o, d);
    int stack[kTraversalStack];
    int sp = 0;
    int node = 0;
    while (true) {
        if (node >= 0) {
            DNode n = load_node(nodes, node);
            if (kCount) cnt->nodes++;
            float t0, t1;
            int m = box2(n, rp, tnear, tfar, t0, t1);
            if (m == 3) {
                int nearC = n.d.x, farC = n.d.y;
                if (t1 < t0) {
                    nearC = n.d.y;
                    farC = n.d.x;
                }
                if (sp < kTraversalStack) {
                    stack[sp++] = farC;
                } else {
                    atomicOr(status, kStatusStackOverflow);
                }
                node = nearC;
                continue;
            } else if (m == 1) {
                node = n.d.x;
                continue;
            } else if (m == 2) {
                node = n.d.y;
                continue;
            }
        } else {
            const int ref = ~node;
            const int last = (ref >> 3) + (ref & 7);
            for (int slot = ref >> 3; slot <= last; ++slot) {
                DTri T = load_tri(tris, slot);
                if (kCount) cnt->tris++;
                float t;
                if (tri_test(T, o, d, tnear, tfar, t)) return true;
            }
        }
        if (sp == 0) break;
        node = stack[--sp];
    }
    return false;
}

// Geometric normal of a hit, normalised and faceforwarded against the ray
// (src/arch/cpu.cpp:76-85; kernel.cu:86-97).
__device__ __forceinline__ f3 hit_normal(const DTri &T, f3 d) {
    f3 e1 = mk3(T.e1.x, T.e1.y, T.e1.z);
    f3 e2 = mk3(T.e2.x, T.e2.y, T.e2.z);
    f3 n = nrmz3(crs3(e1, e2));
    if (dot3(n, d) > 0.f) n = neg3(n);
    return n;
}

}  // namespace hsr
