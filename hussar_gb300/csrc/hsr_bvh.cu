// Device BVH build: replaces Embree's rtcCommitScene (libhussar/src/arch/cpu.cpp:32-47)
// and OptiX's optixAccelBuild + compaction (src/arch/gpu.cpp:82-207).
//
//   1. per-triangle bounds and centroids, scene centroid bounds (k_bounds)
//   2. 63-bit Morton code of each centroid, 21 bits per axis (k_morton)
//   3. radix sort of (code, triangle id) pairs (CUB DeviceRadixSort)
//   4. triangle records written in sorted order (k_write_tris)
//   5. topology, one of:
//      PLOC (default): parallel locally-ordered clustering over the Morton order
//        (Meister and Bittner 2018): every cluster finds, within +-256 positions, the
//        neighbour whose merged box has the smallest surface area; mutual nearest pairs
//        merge; survivors are compacted in order; repeat until one cluster is left.
//        Surface-area-driven like an SAH build, robust to large overlapping triangles.
//      LBVH: binary radix tree from the sorted codes (Karras 2012, k_karras) and a
//        bottom-up box refit (k_refit).
//   6. insertion passes (up to 32, hsr_set_bvh_optimize): every subtree is re-placed in
//      parallel where the surface-area cost falls most (k_reins_*, below)
//   7. leaves: a bottom-up surface-area cost pass turns subtrees of at most the leaf size
//      (default 4, hsr_set_bvh_leaf_size) into leaves when testing their triangles is
//      cheaper than visiting their nodes (k_leaf_cost); the triangle records are reordered so that every
//      leaf's triangles are contiguous (k_leaf_group, radix sort, k_permute_tris) and
//      the links of the remaining nodes rewritten (k_relink).
//   8. the reachable nodes renumbered depth first and the array shrunk to them (host).
// Node i stores the boxes of both its children; node 0 is the root. A child reference
// c >= 0 is an internal node; c < 0 a leaf of ((~c) & 7) + 1 triangles from slot
// (~c) >> 3. A node's first child, when internal, is node i + 1.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_select.cuh>

#include <limits>
#include <vector>

#include "hsr_common.cuh"
#include "hsr_internal.h"

namespace hsr {

namespace {

__device__ __forceinline__ unsigned f2ord(float f) {
    unsigned u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(unsigned u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// Triangle AABB, padded so the FMA slab test stays conservative.
__global__ void k_bounds(const float *__restrict__ v, const int32_t *__restrict__ idx, int64_t nt, float *__restrict__ lo,
                         float *__restrict__ hi, unsigned *__restrict__ cbounds) {
    int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (t >= nt) return;
    float c[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float x0 = v[3 * int64_t(idx[3 * t + 0]) + a];
        float x1 = v[3 * int64_t(idx[3 * t + 1]) + a];
        float x2 = v[3 * int64_t(idx[3 * t + 2]) + a];
        float mn = fminf(x0, fminf(x1, x2)), mx = fmaxf(x0, fmaxf(x1, x2));
        float pad = fmaxf(fabsf(mn), fabsf(mx)) * 4e-6f + 1e-6f;
        lo[3 * t + a] = mn - pad;
        hi[3 * t + a] = mx + pad;
        c[a] = 0.5f * mn + 0.5f * mx;
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        atomicMin(&cbounds[a], f2ord(c[a]));
        atomicMax(&cbounds[3 + a], f2ord(c[a]));
    }
}

__device__ __forceinline__ uint64_t expand21(uint64_t x) {
    x &= 0x1fffffull;
    x = (x | x << 32) & 0x1f00000000ffffull;
    x = (x | x << 16) & 0x1f0000ff0000ffull;
    x = (x | x << 8) & 0x100f00f00f00f00full;
    x = (x | x << 4) & 0x10c30c30c30c30c3ull;
    x = (x | x << 2) & 0x1249249249249249ull;
    return x;
}

__global__ void k_morton(const float *__restrict__ lo, const float *__restrict__ hi, int64_t nt,
                         const unsigned *__restrict__ cbounds, uint64_t *__restrict__ keys, int32_t *__restrict__ ids) {
    int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (t >= nt) return;
    uint64_t code = 0;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float cmin = ord2f(cbounds[a]), cmax = ord2f(cbounds[3 + a]);
        float c = 0.5f * lo[3 * t + a] + 0.5f * hi[3 * t + a];
        float ext = cmax - cmin;
        float u = ext > 0.f ? (c - cmin) / ext : 0.5f;
        u = fminf(fmaxf(u, 0.f), 1.f);
        uint64_t q = uint64_t(fminf(u * 2097152.f, 2097151.f));
        code |= expand21(q) << (2 - a);
    }
    keys[t] = code;
    ids[t] = int32_t(t);
}

__global__ void k_write_tris(const float *__restrict__ v, const int32_t *__restrict__ idx,
                             const int32_t *__restrict__ sorted_ids, int64_t nt, DTri *__restrict__ tris) {
    int64_t s = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (s >= nt) return;
    int64_t t = sorted_ids[s];
    const float *p0 = v + 3 * int64_t(idx[3 * t + 0]);
    const float *p1 = v + 3 * int64_t(idx[3 * t + 1]);
    const float *p2 = v + 3 * int64_t(idx[3 * t + 2]);
    DTri T;
    T.v0 = make_float4(p0[0], p0[1], p0[2], __int_as_float(int(t)));
    T.e1 = make_float4(p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2], 0.f);
    T.e2 = make_float4(p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2], 0.f);
    tris[s] = T;
}

// common prefix length of sorted keys i and j, with the index as a tie-breaker
__device__ __forceinline__ int delta(const uint64_t *__restrict__ k, int64_t n, int64_t i, int64_t j) {
    if (j < 0 || j >= n) return -1;
    uint64_t a = k[i], b = k[j];
    if (a == b) return 64 + __clzll((unsigned long long)(i ^ j));
    return __clzll((unsigned long long)(a ^ b));
}

// Karras 2012: internal node i covers a key range; its split is the highest differing bit.
__global__ void k_karras(const uint64_t *__restrict__ k, int64_t n, DNode *__restrict__ nodes,
                         int32_t *__restrict__ parent_internal, int32_t *__restrict__ parent_leaf) {
    int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= n - 1) return;
    int d = (delta(k, n, i, i + 1) - delta(k, n, i, i - 1)) >= 0 ? 1 : -1;
    int dmin = delta(k, n, i, i - d);
    int64_t lmax = 2;
    while (delta(k, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int64_t l = 0;
    for (int64_t t = lmax >> 1; t >= 1; t >>= 1)
        if (delta(k, n, i, i + (l + t) * d) > dmin) l += t;
    int64_t j = i + l * d;
    int dnode = delta(k, n, i, j);
    int64_t s = 0;
    int64_t len = l;
    int64_t t = (len + 1) >> 1;
    while (true) {
        if (delta(k, n, i, i + (s + t) * d) > dnode) s += t;
        if (t == 1) break;
        t = (t + 1) >> 1;
    }
    int64_t gamma = i + s * d + (d < 0 ? -1 : 0);
    int64_t first = i < j ? i : j, last = i < j ? j : i;
    int c0, c1;
    if (first == gamma) {
        c0 = ~int(gamma);
        parent_leaf[gamma] = int(i);
    } else {
        c0 = int(gamma);
        parent_internal[gamma] = int(i);
    }
    if (last == gamma + 1) {
        c1 = ~int(gamma + 1);
        parent_leaf[gamma + 1] = int(i);
    } else {
        c1 = int(gamma + 1);
        parent_internal[gamma + 1] = int(i);
    }
    nodes[i].d = make_int4(c0, c1, 0, 0);
}

struct Box {
    float lo[3], hi[3];
};

__device__ __forceinline__ Box child_box(const DNode &n, int which) {
    Box b;
    if (which == 0) {
        b.lo[0] = n.a.x; b.hi[0] = n.a.y; b.lo[1] = n.a.z; b.hi[1] = n.a.w; b.lo[2] = n.c.x; b.hi[2] = n.c.y;
    } else {
        b.lo[0] = n.b.x; b.hi[0] = n.b.y; b.lo[1] = n.b.z; b.hi[1] = n.b.w; b.lo[2] = n.c.z; b.hi[2] = n.c.w;
    }
    return b;
}

// Bottom-up refit: a leaf's thread climbs while it is the second child to arrive.
__global__ void k_refit(int64_t n, const int32_t *__restrict__ sorted_ids, const float *__restrict__ lo,
                        const float *__restrict__ hi, DNode *nodes, const int32_t *__restrict__ parent_internal,
                        const int32_t *__restrict__ parent_leaf, int *counters, int *depth_out) {
    int64_t leaf = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (leaf >= n) return;
    int p = parent_leaf[leaf];
    int depth = 1;
    while (p >= 0) {
        __threadfence();
        int prev = atomicAdd(&counters[p], 1);
        if (prev == 0) return;  // the sibling subtree is not finished; its thread continues
        __threadfence();
        volatile DNode *vn = nodes;
        int c[2] = {vn[p].d.x, vn[p].d.y};
        Box bx[2];
        for (int w = 0; w < 2; ++w) {
            if (c[w] < 0) {
                int64_t t = sorted_ids[~c[w]];
                for (int a = 0; a < 3; ++a) {
                    bx[w].lo[a] = lo[3 * t + a];
                    bx[w].hi[a] = hi[3 * t + a];
                }
            } else {
                DNode cn;
                cn.a = make_float4(vn[c[w]].a.x, vn[c[w]].a.y, vn[c[w]].a.z, vn[c[w]].a.w);
                cn.b = make_float4(vn[c[w]].b.x, vn[c[w]].b.y, vn[c[w]].b.z, vn[c[w]].b.w);
                cn.c = make_float4(vn[c[w]].c.x, vn[c[w]].c.y, vn[c[w]].c.z, vn[c[w]].c.w);
                Box b0 = child_box(cn, 0), b1 = child_box(cn, 1);
                for (int a = 0; a < 3; ++a) {
                    bx[w].lo[a] = fminf(b0.lo[a], b1.lo[a]);
                    bx[w].hi[a] = fmaxf(b0.hi[a], b1.hi[a]);
                }
            }
        }
        vn[p].a.x = bx[0].lo[0]; vn[p].a.y = bx[0].hi[0]; vn[p].a.z = bx[0].lo[1]; vn[p].a.w = bx[0].hi[1];
        vn[p].b.x = bx[1].lo[0]; vn[p].b.y = bx[1].hi[0]; vn[p].b.z = bx[1].lo[1]; vn[p].b.w = bx[1].hi[1];
        vn[p].c.x = bx[0].lo[2]; vn[p].c.y = bx[0].hi[2]; vn[p].c.z = bx[1].lo[2]; vn[p].c.w = bx[1].hi[2];
        p = parent_internal[p];
        depth++;
    }
    atomicMax(depth_out, depth);
}

// Leaf depth statistics: each leaf walks to the root.
__global__ void k_leaf_depth(int64_t n, const int32_t *__restrict__ parent_internal,
                             const int32_t *__restrict__ parent_leaf, int *depth_out) {
    int64_t leaf = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (leaf >= n) return;
    int p = parent_leaf[leaf];
    int depth = 1;
    while (p >= 0 && depth < 1 << 20) {
        p = parent_internal[p];
        depth++;
    }
    atomicMax(depth_out, depth);
}

// ---------------- PLOC ----------------
constexpr int kPlocRadius = 256;

struct Cluster {
    int id;       // node encoding: >= 0 internal node, < 0 leaf slot (~slot)
    float b[6];   // lo.xyz, hi.xyz
};

__global__ void k_ploc_init(int64_t n, const int32_t *__restrict__ sorted_ids, const float *__restrict__ lo,
                            const float *__restrict__ hi, Cluster *__restrict__ cl) {
    int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= n) return;
    const int64_t t = sorted_ids[i];
    Cluster c;
    c.id = ~int(i);
    for (int a = 0; a < 3; ++a) {
        c.b[a] = lo[3 * t + a];
        c.b[3 + a] = hi[3 * t + a];
    }
    cl[i] = c;
}

__device__ __forceinline__ float merged_area(const float *a, const float *b) {
    const float dx = fmaxf(a[3], b[3]) - fminf(a[0], b[0]);
    const float dy = fmaxf(a[4], b[4]) - fminf(a[1], b[1]);
    const float dz = fmaxf(a[5], b[5]) - fminf(a[2], b[2]);
    return dx * dy + dy * dz + dz * dx;
}

// nearest[i]: the cluster within +-R whose union with i has the smallest surface area
// (ties: the lower index), read through a shared-memory window.
__global__ void __launch_bounds__(256) k_ploc_nearest(int n, const Cluster *__restrict__ cl, int *__restrict__ nearest) {
    __shared__ float sb[256 + 2 * kPlocRadius][6];
    const int base = blockIdx.x * 256;
    for (int k = threadIdx.x; k < 256 + 2 * kPlocRadius; k += 256) {
        const int j = base - kPlocRadius + k;
        if (j >= 0 && j < n) {
#pragma unroll
            for (int a = 0; a < 6; ++a) sb[k][a] = cl[j].b[a];
        }
    }
    __syncthreads();
    const int i = base + threadIdx.x;
    if (i >= n) return;
    const float *bi = sb[threadIdx.x + kPlocRadius];
    float best = __int_as_float(0x7f800000);
    int bj = -1;
    const int j0 = max(0, i - kPlocRadius), j1 = min(n - 1, i + kPlocRadius);
    for (int j = j0; j <= j1; ++j) {
        if (j == i) continue;
        const float a = merged_area(bi, sb[j - base + kPlocRadius]);
        if (a < best) {
            best = a;
            bj = j;
        }
    }
    nearest[i] = bj;
}

// Mutual nearest pairs merge into a new internal node (allocated from the top so that the
// last merge, the root, is node 0); the lower index keeps the merged cluster.
__global__ void k_ploc_merge(int n, const int *__restrict__ nearest, Cluster *cl, char *__restrict__ keep,
                             DNode *__restrict__ nodes, int *__restrict__ node_counter, int internal_total,
                             int32_t *__restrict__ parent_internal, int32_t *__restrict__ parent_leaf) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int j = nearest[i];
    if (j < 0 || nearest[j] != i) {
        keep[i] = 1;
        return;
    }
    if (i > j) {
        keep[i] = 0;
        return;
    }
    const Cluster a = cl[i], b = cl[j];
    const int id = internal_total - 1 - atomicAdd(node_counter, 1);
    DNode nd;
    nd.a = make_float4(a.b[0], a.b[3], a.b[1], a.b[4]);
    nd.b = make_float4(b.b[0], b.b[3], b.b[1], b.b[4]);
    nd.c = make_float4(a.b[2], a.b[5], b.b[2], b.b[5]);
    nd.d = make_int4(a.id, b.id, 0, 0);
    nodes[id] = nd;
    if (a.id >= 0) parent_internal[a.id] = id; else parent_leaf[~a.id] = id;
    if (b.id >= 0) parent_internal[b.id] = id; else parent_leaf[~b.id] = id;
    Cluster m;
    m.id = id;
    for (int k = 0; k < 3; ++k) {
        m.b[k] = fminf(a.b[k], b.b[k]);
        m.b[3 + k] = fmaxf(a.b[3 + k], b.b[3 + k]);
    }
    cl[i] = m;
    keep[i] = 1;
}

inline unsigned blocks_for(int64_t n, int t) { return unsigned((n + t - 1) / t); }

// ---------------- leaves of several triangles ----------------
// Costs of the leaf decision per unit of a node's surface area: one node visit (two child
// boxes, 64 bytes) and one triangle test (48 bytes and the Moller-Trumbore arithmetic with
// its divide). Measured with leaves of up to 4: a triangle test costing 1 node visit made
// the boxes workload 6 % slower than one triangle per leaf, 2 made it 2 % faster, 3 and 4
// 3 % faster (urban +6 %, sphere +7 %).
constexpr float kCostNode = 1.0f;
constexpr float kCostTri = 3.0f;

__device__ __forceinline__ float box_area(const Box &b) {
    const float dx = b.hi[0] - b.lo[0], dy = b.hi[1] - b.lo[1], dz = b.hi[2] - b.lo[2];
    return dx * dy + dy * dz + dz * dx;
}

// Bottom-up (a leaf's thread climbs while it is the second child to arrive): per node the
// triangle count and the cheaper of its two costs; a node (not the root) whose triangles
// fit a leaf and cost no more as one is marked collapsible.
__global__ void k_leaf_cost(int64_t n, const DNode *__restrict__ nodes, const int32_t *__restrict__ parent_internal,
                            const int32_t *__restrict__ parent_leaf, int *counters, int *count, float *cost,
                            char *collapse, int leaf_max) {
    const int64_t leaf = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (leaf >= n) return;
    int p = parent_leaf[leaf];
    while (p >= 0) {
        __threadfence();
        if (atomicAdd(&counters[p], 1) == 0) return;  // the sibling's thread continues
        __threadfence();
        const DNode nd = nodes[p];
        const int c[2] = {nd.d.x, nd.d.y};
        const volatile int *vcount = count;
        const volatile float *vcost = cost;
        int cnt = 0;
        float sum = 0.f;
        Box u;
        for (int w = 0; w < 2; ++w) {
            const Box b = child_box(nd, w);
            const int cc = c[w] < 0 ? 1 : vcount[c[w]];
            const float cw = c[w] < 0 ? kCostTri : vcost[c[w]];
            cnt += cc;
            sum += box_area(b) * cw;
            for (int a = 0; a < 3; ++a) {
                u.lo[a] = w ? fminf(u.lo[a], b.lo[a]) : b.lo[a];
                u.hi[a] = w ? fmaxf(u.hi[a], b.hi[a]) : b.hi[a];
            }
        }
        const float area = box_area(u);
        const float as_node = kCostNode + (area > 0.f ? sum / area : 0.f);
        const float as_leaf = kCostTri * float(cnt);
        const bool leafy = p != 0 && cnt <= leaf_max && as_leaf <= as_node;
        count[p] = cnt;
        cost[p] = leafy ? as_leaf : as_node;
        collapse[p] = leafy ? 1 : 0;
        p = parent_internal[p];
    }
}

// Per triangle slot: the topmost collapsible ancestor within the leaf-sized part of the
// tree above it (-1: a leaf of its own), and the group's smallest slot.
__global__ void k_leaf_group(int64_t n, const int32_t *__restrict__ parent_internal,
                             const int32_t *__restrict__ parent_leaf, const int *__restrict__ count,
                             const char *__restrict__ collapse, int leaf_max, int32_t *__restrict__ group,
                             int *__restrict__ group_min, char *__restrict__ is_root) {
    const int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (t >= n) return;
    int p = parent_leaf[t], root = -1;
    while (p >= 0 && count[p] <= leaf_max) {
        if (collapse[p]) root = p;
        p = parent_internal[p];
    }
    group[t] = root;
    if (root >= 0) {
        atomicMin(&group_min[root], int(t));
        is_root[root] = 1;
    }
}

// sort key: the group's smallest slot, then the slot (groups stay in the Morton order)
__global__ void k_leaf_keys(int64_t n, const int32_t *__restrict__ group, const int *__restrict__ group_min,
                            uint64_t *__restrict__ keys, int32_t *__restrict__ ids) {
    const int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (t >= n) return;
    const uint64_t g = group[t] >= 0 ? uint64_t(group_min[group[t]]) : uint64_t(t);
    keys[t] = (g << 32) | uint64_t(t);
    ids[t] = int32_t(t);
}

// new slot of every old slot; records moved; each group's first new slot
__global__ void k_permute_tris(int64_t n, const int32_t *__restrict__ sorted_old, const DTri *__restrict__ src,
                               DTri *__restrict__ dst, int32_t *__restrict__ new_slot) {
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= n) return;
    const int32_t old = sorted_old[i];
    dst[i] = src[old];
    new_slot[old] = int32_t(i);
}

__global__ void k_leaf_start(int64_t n, const int32_t *__restrict__ group, const int32_t *__restrict__ new_slot,
                             int *__restrict__ start) {
    const int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (t >= n || group[t] < 0) return;
    atomicMin(&start[group[t]], new_slot[t]);
}

// child references in the leaf encoding: a collapsed subtree becomes its leaf, a single
// triangle moves to its new slot
__global__ void k_relink(int64_t n_nodes, DNode *nodes, const int32_t *__restrict__ new_slot,
                         const char *__restrict__ is_root, const int *__restrict__ start,
                         const int *__restrict__ count) {
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= n_nodes) return;
    int c[2] = {nodes[i].d.x, nodes[i].d.y};
    for (int w = 0; w < 2; ++w) {
        if (c[w] < 0)
            c[w] = ~(new_slot[~c[w]] << 3);
        else if (is_root[c[w]])
            c[w] = ~((start[c[w]] << 3) | (count[c[w]] - 1));
    }
    nodes[i].d.x = c[0];
    nodes[i].d.y = c[1];
}

// ---------------- insertion-based optimisation ----------------
// Bittner, Hapala and Havran (2013): take a subtree out and insert it as the sibling of
// the node where the tree's surface-area cost grows least. Every node searches in
// parallel on a snapshot of the tree (Meister and Bittner 2018); the moves that lower the
// cost claim the six nodes they rewire (the subtree N, its parent P and sibling S, its
// grandparent G, the target X and X's parent) with 64-bit priority locks (gain, node); a
// winner whose target lies inside another winner's subtree withdraws, so no move closes a
// cycle; the winners are applied and the boxes refitted. Index space: internal nodes
// [0, M), triangle slot t at M + t. The root stays node 0 (never moved, never a target,
// never removed). The build's DNodes are written back only when the result passes its
// checks (every node's parent chain ends at node 0; leaves at most 60 deep).
constexpr int kReinsPath = 96;       // deepest parent chain a search handles
constexpr int kReinsHeap = 384;      // search frontier (a fuller frontier drops entries)
constexpr int kReinsPops = 4096;
constexpr int kReinsMaxDepth = 60;   // the traversal stack holds 64 entries

__device__ __forceinline__ Box box_union(const Box &a, const Box &b) {
    Box u;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        u.lo[k] = fminf(a.lo[k], b.lo[k]);
        u.hi[k] = fmaxf(a.hi[k], b.hi[k]);
    }
    return u;
}

__global__ void k_reins_init(int m, const DNode *__restrict__ nodes, const int32_t *__restrict__ par_i, int *rpar,
                             int2 *rkid, Box *rbox) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const DNode nd = nodes[i];
    const int c[2] = {nd.d.x, nd.d.y};
    int k[2];
    for (int w = 0; w < 2; ++w) {
        k[w] = c[w] >= 0 ? c[w] : m + ~c[w];
        if (c[w] < 0) {
            rbox[k[w]] = child_box(nd, w);
            rpar[k[w]] = i;
        }
    }
    rkid[i] = make_int2(k[0], k[1]);
    rpar[i] = par_i[i];
    rbox[i] = box_union(child_box(nd, 0), child_box(nd, 1));
}

// Depth of every node (the root 0) and the deepest leaf; bad: a parent chain that does not
// end at node 0 within the bound.
__global__ void k_reins_depth(int total, int m, const int *__restrict__ rpar, int *depth, int *max_depth,
                              int *bad) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    int d = 0, x = i;
    while (rpar[x] >= 0 && d < 1024) {
        x = rpar[x];
        ++d;
    }
    depth[i] = d;
    if (x != 0 || d >= 1024) atomicOr(bad, 1);
    if (i >= m) atomicMax(max_depth, d);
}

// The best place for subtree n: mv_x[n] (-1: none lowers the cost by min_gain) and the
// cost it saves, mv_gain[n].
__global__ void __launch_bounds__(128) k_reins_search(int total, int m, const int *__restrict__ rpar,
                                                      const int2 *__restrict__ rkid, const Box *__restrict__ rbox,
                                                      const int *__restrict__ depth, float min_gain, int *mv_x,
                                                      float *mv_gain) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= total) return;
    mv_x[n] = -1;
    const int P = rpar[n];
    if (P < 0) return;
    const int G = rpar[P];
    if (G < 0) return;
    const int dp = depth[P];
    if (dp >= kReinsPath) return;
    const int2 pk = rkid[P];
    const int S = pk.x == n ? pk.y : pk.x;
    // the tree with n taken out: P disappears, S takes its place, P's ancestors shrink
    int pnode[kReinsPath];
    Box pbox[kReinsPath];
    float drem = -box_area(rbox[P]);
    Box cur = rbox[S];
    int child = P;
    for (int y = G, steps = 0; y >= 0; child = y, y = rpar[y], ++steps) {
        const int dy = depth[y];
        if (steps >= kReinsPath || dy < 0 || dy >= dp) return;  // an inconsistent snapshot: no move
        const int2 yk = rkid[y];
        const Box nb = box_union(cur, rbox[yk.x == child ? yk.y : yk.x]);
        drem += box_area(nb) - box_area(rbox[y]);
        pnode[dy] = y;
        pbox[dy] = nb;
        cur = nb;
    }
    const Box bn = rbox[n];
    const float an = box_area(bn);
    // best-first branch and bound over the detached tree; a node's key is the area its
    // ancestors grow by when n goes below them (the induced cost). Only a place whose
    // insertion cost is below -drem - min_gain saves more than min_gain: that is the
    // starting bound, so a subtree already well placed ends its search at once.
    float hk[kReinsHeap];
    int hv[kReinsHeap];
    int hs = 1;
    hk[0] = 0.f;
    hv[0] = 0;
    float best = -drem - min_gain;
    int bx = -1;
    for (int pops = 0; hs > 0 && pops < kReinsPops; ++pops) {
        const float ic0 = hk[0];
        int x = hv[0];
        --hs;
        if (hs > 0) {  // sift the last entry down from the top
            const float k = hk[hs];
            const int v = hv[hs];
            int i = 0;
            while (true) {
                int c = 2 * i + 1;
                if (c >= hs) break;
                if (c + 1 < hs && hk[c + 1] < hk[c]) ++c;
                if (hk[c] >= k) break;
                hk[i] = hk[c];
                hv[i] = hv[c];
                i = c;
            }
            hk[i] = k;
            hv[i] = v;
        }
        if (ic0 + an >= best) break;
        if (x == P) x = S;
        const int dx = depth[x];
        const Box bxx = (dx < dp && pnode[dx] == x) ? pbox[dx] : rbox[x];
        const float au = box_area(box_union(bxx, bn));
        if (x != S && x != 0 && ic0 + au < best) {
            best = ic0 + au;
            bx = x;
        }
        const float ic = ic0 + au - box_area(bxx);
        if (x < m && ic + an < best) {
            const int2 xk = rkid[x];
            for (int w = 0; w < 2; ++w) {
                if (hs >= kReinsHeap) break;
                int i = hs++;
                while (i > 0 && hk[(i - 1) / 2] > ic) {
                    hk[i] = hk[(i - 1) / 2];
                    hv[i] = hv[(i - 1) / 2];
                    i = (i - 1) / 2;
                }
                hk[i] = ic;
                hv[i] = w ? xk.y : xk.x;
            }
        }
    }
    const float gain = -(drem + best);
    if (bx >= 0 && gain > min_gain) {  // bx >= 0 already means gain > min_gain, up to rounding
        mv_x[n] = bx;
        mv_gain[n] = gain;
    }
}

// The nodes a move rewires: n, P, S, G, X, X's parent.
__device__ __forceinline__ void reins_touched(int n, int x, const int *rpar, const int2 *rkid, int *t) {
    const int P = rpar[n];
    const int2 pk = rkid[P];
    t[0] = n;
    t[1] = P;
    t[2] = pk.x == n ? pk.y : pk.x;
    t[3] = rpar[P];
    t[4] = x;
    t[5] = rpar[x];
}

__global__ void k_reins_lock(int total, const int *__restrict__ rpar, const int2 *__restrict__ rkid,
                             const int *__restrict__ mv_x, const float *__restrict__ mv_gain,
                             unsigned long long *lock) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= total || mv_x[n] < 0) return;
    int t[6];
    reins_touched(n, mv_x[n], rpar, rkid, t);
    for (int k = 0; k < 6; ++k)
        if (t[k] < 0 || t[k] >= total) return;
    const unsigned long long key = (static_cast<unsigned long long>(__float_as_uint(mv_gain[n])) << 32) | unsigned(n);
    for (int k = 0; k < 6; ++k) atomicMax(&lock[t[k]], key);
}

__global__ void k_reins_claim(int total, const int *__restrict__ rpar, const int2 *__restrict__ rkid,
                              const int *__restrict__ mv_x, const float *__restrict__ mv_gain,
                              const unsigned long long *__restrict__ lock, char *moving) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= total) return;
    moving[n] = 0;
    if (mv_x[n] < 0) return;
    int t[6];
    reins_touched(n, mv_x[n], rpar, rkid, t);
    const unsigned long long key = (static_cast<unsigned long long>(__float_as_uint(mv_gain[n])) << 32) | unsigned(n);
    for (int k = 0; k < 6; ++k)
        if (t[k] < 0 || t[k] >= total || lock[t[k]] != key) return;
    moving[n] = 1;
}

// A winner stays unless its target is inside another winner's subtree.
__global__ void k_reins_keep(int total, const int *__restrict__ rpar, const int *__restrict__ mv_x,
                             const char *__restrict__ moving, char *keep) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= total) return;
    keep[n] = 0;
    if (!moving[n]) return;
    int x = mv_x[n];
    for (int steps = 0; x >= 0; x = rpar[x], ++steps)
        if (steps >= 1024 || (x != n && moving[x])) return;
    keep[n] = 1;
}

__global__ void k_reins_apply(int total, int *rpar, int2 *rkid, const int *__restrict__ mv_x,
                              const char *__restrict__ keep, int *applied) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= total || !keep[n]) return;
    const int X = mv_x[n];
    const int P = rpar[n], G = rpar[P];
    const int2 pk = rkid[P];
    const int S = pk.x == n ? pk.y : pk.x;
    // take n out: S replaces P below G
    int2 gk = rkid[G];
    if (gk.x == P) gk.x = S; else gk.y = S;
    rkid[G] = gk;
    rpar[S] = G;
    // P becomes the parent of X and n, in X's place
    const int XP = rpar[X];
    int2 xk = rkid[XP];
    if (xk.x == X) xk.x = P; else xk.y = P;
    rkid[XP] = xk;
    rpar[P] = XP;
    rkid[P] = make_int2(X, n);
    rpar[X] = P;
    rpar[n] = P;
    atomicAdd(applied, 1);
}

// Boxes from the leaves up: a leaf's thread climbs while it is the second child to arrive.
__global__ void k_reins_refit(int total, int m, const int *__restrict__ rpar, const int2 *__restrict__ rkid,
                              Box *rbox, int *counters, int *bad) {
    const int leaf = m + blockIdx.x * blockDim.x + threadIdx.x;
    if (leaf >= total) return;
    int p = rpar[leaf];
    for (int steps = 0; p >= 0; p = rpar[p], ++steps) {
        if (steps >= 1024) {
            atomicOr(bad, 1);
            return;
        }
        __threadfence();
        if (atomicAdd(&counters[p], 1) == 0) return;
        __threadfence();
        const int2 k = rkid[p];
        const volatile Box *vb = rbox;
        Box a, b;
        for (int j = 0; j < 3; ++j) {
            a.lo[j] = vb[k.x].lo[j];
            a.hi[j] = vb[k.x].hi[j];
            b.lo[j] = vb[k.y].lo[j];
            b.hi[j] = vb[k.y].hi[j];
        }
        rbox[p] = box_union(a, b);
    }
}

// Back to the build's layout: DNodes with child boxes and references (leaf: ~slot),
// internal and leaf parent links.
__global__ void k_reins_write(int m, const int *__restrict__ rpar, const int2 *__restrict__ rkid,
                              const Box *__restrict__ rbox, DNode *nodes, int32_t *par_i, int32_t *par_l) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const int2 k = rkid[i];
    const Box l = rbox[k.x], r = rbox[k.y];
    DNode nd;
    nd.a = make_float4(l.lo[0], l.hi[0], l.lo[1], l.hi[1]);
    nd.b = make_float4(r.lo[0], r.hi[0], r.lo[1], r.hi[1]);
    nd.c = make_float4(l.lo[2], l.hi[2], r.lo[2], r.hi[2]);
    nd.d = make_int4(k.x < m ? k.x : ~(k.x - m), k.y < m ? k.y : ~(k.y - m), 0, 0);
    nodes[i] = nd;
    par_i[i] = rpar[i];
    if (k.x >= m) par_l[k.x - m] = i;
    if (k.y >= m) par_l[k.y - m] = i;
}

}  // namespace

int g_bvh_builder = 0;  // 0: PLOC, 1: LBVH (Karras)
int g_bvh_leaf_max = 4;  // triangles per leaf (1..8)
int g_bvh_optimize = 32;  // largest number of insertion passes after the build (0: none)

// Insertion passes over the binary tree of a build (par_i/par_l and the DNodes, leaves
// referenced as ~slot); stops when a pass moves fewer than 1 in 20,000 nodes (stopping
// at 1 in 4,000 left the urban scene 8 % more node visits per ray). Returns 0
// (also when the result failed its checks and the build's tree was kept), 2 or 3.
static int optimize_tree(SceneDev &s, int64_t nt, int32_t *par_i, int32_t *par_l, cudaStream_t st,
                         std::string &err) {
    if (g_bvh_optimize <= 0 || nt < 4 || nt >= (int64_t(1) << 30)) return 0;
    const int m = int(nt - 1), total = int(2 * nt - 1);
    int *rpar = nullptr, *depth = nullptr, *mv_x = nullptr, *counters = nullptr, *scal = nullptr;
    int2 *rkid = nullptr;
    Box *rbox = nullptr;
    float *mv_gain = nullptr;
    unsigned long long *lock = nullptr;
    char *moving = nullptr, *keep = nullptr;
    int rc = 0;
    do {
        if (!dev_alloc(&rpar, sizeof(int) * total, err) || !dev_alloc(&depth, sizeof(int) * total, err) ||
            !dev_alloc(&mv_x, sizeof(int) * total, err) || !dev_alloc(&counters, sizeof(int) * m, err) ||
            !dev_alloc(&scal, sizeof(int) * 4, err) || !dev_alloc(&rkid, sizeof(int2) * m, err) ||
            !dev_alloc(&rbox, sizeof(Box) * total, err) || !dev_alloc(&mv_gain, sizeof(float) * total, err) ||
            !dev_alloc(&lock, sizeof(unsigned long long) * total, err) || !dev_alloc(&moving, size_t(total), err) ||
            !dev_alloc(&keep, size_t(total), err)) {
            rc = 3;
            break;
        }
        const int T = 256;
        k_reins_init<<<blocks_for(m, T), T, 0, st>>>(m, s.nodes, par_i, rpar, rkid, rbox);
        note_launches(1);
        Box root;
        if (cudaMemcpyAsync(&root, rbox, sizeof(Box), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess) {
            err = "BVH optimisation: reading the root box failed";
            rc = 2;
            break;
        }
        const float dx = root.hi[0] - root.lo[0], dy = root.hi[1] - root.lo[1], dz = root.hi[2] - root.lo[2];
        const float min_gain = 1e-6f * (dx * dy + dy * dz + dz * dx);
        int h[4] = {0, 0, 0, 0};
        for (int pass = 0; pass < g_bvh_optimize; ++pass) {
            cudaMemsetAsync(scal, 0, sizeof(int) * 4, st);
            cudaMemsetAsync(lock, 0, sizeof(unsigned long long) * total, st);
            cudaMemsetAsync(counters, 0, sizeof(int) * m, st);
            k_reins_depth<<<blocks_for(total, T), T, 0, st>>>(total, m, rpar, depth, scal + 2, scal + 1);
            k_reins_search<<<blocks_for(total, 128), 128, 0, st>>>(total, m, rpar, rkid, rbox, depth, min_gain, mv_x,
                                                                   mv_gain);
            k_reins_lock<<<blocks_for(total, T), T, 0, st>>>(total, rpar, rkid, mv_x, mv_gain, lock);
            k_reins_claim<<<blocks_for(total, T), T, 0, st>>>(total, rpar, rkid, mv_x, mv_gain, lock, moving);
            k_reins_keep<<<blocks_for(total, T), T, 0, st>>>(total, rpar, mv_x, moving, keep);
            k_reins_apply<<<blocks_for(total, T), T, 0, st>>>(total, rpar, rkid, mv_x, keep, scal);
            k_reins_refit<<<blocks_for(nt, T), T, 0, st>>>(total, m, rpar, rkid, rbox, counters, scal + 1);
            note_launches(7);
            if (cudaMemcpyAsync(h, scal, sizeof(h), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                cudaStreamSynchronize(st) != cudaSuccess) {
                err = "BVH optimisation pass failed";
                rc = 2;
                break;
            }
            if (h[1] || h[0] < std::max(1, total / 20000)) break;
        }
        if (rc || h[1]) break;  // a failed check keeps the build's own tree
        cudaMemsetAsync(scal, 0, sizeof(int) * 4, st);
        k_reins_depth<<<blocks_for(total, T), T, 0, st>>>(total, m, rpar, depth, scal + 2, scal + 1);
        note_launches(1);
        if (cudaMemcpyAsync(h, scal, sizeof(h), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess) {
            err = "BVH optimisation check failed";
            rc = 2;
            break;
        }
        if (h[1] || h[2] > kReinsMaxDepth) break;
        k_reins_write<<<blocks_for(m, T), T, 0, st>>>(m, rpar, rkid, rbox, s.nodes, par_i, par_l);
        note_launches(1);
        if (cudaStreamSynchronize(st) != cudaSuccess) {
            err = "BVH optimisation write-back failed";
            rc = 2;
        }
    } while (false);
    cudaFree(rpar);
    cudaFree(depth);
    cudaFree(mv_x);
    cudaFree(counters);
    cudaFree(scal);
    cudaFree(rkid);
    cudaFree(rbox);
    cudaFree(mv_gain);
    cudaFree(lock);
    cudaFree(moving);
    cudaFree(keep);
    return rc;
}

// Leaves of several triangles over a built binary topology (parent links of the build).
static int collapse_leaves(SceneDev &s, int64_t nt, const int32_t *par_i, const int32_t *par_l, int *counters,
                           cudaStream_t st, std::string &err) {
    const int64_t n_nodes = s.node_count;
    const int leaf_max = std::min(std::max(g_bvh_leaf_max, 1), 8);
    int *count = nullptr, *group_min = nullptr, *start = nullptr;
    float *cost = nullptr;
    char *collapse = nullptr, *is_root = nullptr;
    int32_t *group = nullptr, *ids = nullptr, *ids2 = nullptr, *new_slot = nullptr;
    uint64_t *keys = nullptr, *keys2 = nullptr;
    DTri *tris2 = nullptr;
    void *tmp = nullptr;
    size_t tmp_bytes = 0;
    int rc = 0;
    do {
        if (!dev_alloc(&count, sizeof(int) * n_nodes, err) || !dev_alloc(&cost, sizeof(float) * n_nodes, err) ||
            !dev_alloc(&collapse, size_t(n_nodes), err) || !dev_alloc(&is_root, size_t(n_nodes), err) ||
            !dev_alloc(&group_min, sizeof(int) * n_nodes, err) || !dev_alloc(&start, sizeof(int) * n_nodes, err) ||
            !dev_alloc(&group, sizeof(int32_t) * nt, err) || !dev_alloc(&ids, sizeof(int32_t) * nt, err) ||
            !dev_alloc(&ids2, sizeof(int32_t) * nt, err) || !dev_alloc(&new_slot, sizeof(int32_t) * nt, err) ||
            !dev_alloc(&keys, sizeof(uint64_t) * nt, err) || !dev_alloc(&keys2, sizeof(uint64_t) * nt, err) ||
            !dev_alloc(&tris2, sizeof(DTri) * nt, err)) {
            rc = 3;
            break;
        }
        cudaMemsetAsync(counters, 0, sizeof(int) * n_nodes, st);
        cudaMemsetAsync(count, 0x7f, sizeof(int) * n_nodes, st);  // > leaf_max until written
        cudaMemsetAsync(collapse, 0, size_t(n_nodes), st);
        cudaMemsetAsync(is_root, 0, size_t(n_nodes), st);
        cudaMemsetAsync(group_min, 0x7f, sizeof(int) * n_nodes, st);
        cudaMemsetAsync(start, 0x7f, sizeof(int) * n_nodes, st);
        const int T = 256;
        if (leaf_max > 1) {
            k_leaf_cost<<<blocks_for(nt, T), T, 0, st>>>(nt, s.nodes, par_i, par_l, counters, count, cost, collapse,
                                                          leaf_max);
            note_launches(1);
        }
        k_leaf_group<<<blocks_for(nt, T), T, 0, st>>>(nt, par_i, par_l, count, collapse, leaf_max, group, group_min,
                                                       is_root);
        k_leaf_keys<<<blocks_for(nt, T), T, 0, st>>>(nt, group, group_min, keys, ids);
        note_launches(2);
        if (cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, keys, keys2, ids, ids2, int(nt), 0, 64, st) !=
                cudaSuccess ||
            !dev_alloc(&tmp, tmp_bytes, err)) {
            if (err.empty()) err = "leaf sort size query failed";
            rc = tmp ? 2 : 3;
            break;
        }
        if (cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, keys, keys2, ids, ids2, int(nt), 0, 64, st) !=
            cudaSuccess) {
            err = "leaf sort failed";
            rc = 2;
            break;
        }
        k_permute_tris<<<blocks_for(nt, T), T, 0, st>>>(nt, ids2, s.tris, tris2, new_slot);
        k_leaf_start<<<blocks_for(nt, T), T, 0, st>>>(nt, group, new_slot, start);
        k_relink<<<blocks_for(n_nodes, T), T, 0, st>>>(n_nodes, s.nodes, new_slot, is_root, start, count);
        note_launches(4);
        const cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            err = std::string("BVH leaves: ") + cudaGetErrorString(e);
            rc = 2;
            break;
        }
        std::swap(s.tris, tris2);
    } while (false);
    cudaFree(count);
    cudaFree(cost);
    cudaFree(collapse);
    cudaFree(is_root);
    cudaFree(group_min);
    cudaFree(start);
    cudaFree(group);
    cudaFree(ids);
    cudaFree(ids2);
    cudaFree(new_slot);
    cudaFree(keys);
    cudaFree(keys2);
    cudaFree(tris2);
    cudaFree(tmp);
    return rc;
}

// PLOC topology over the sorted leaves. Returns 0 or an hsr_status-like code.
static int build_ploc(SceneDev &s, int64_t nt, const int32_t *ids2, const float *lo, const float *hi,
                      int32_t *par_i, int32_t *par_l, int *depth, cudaStream_t st, std::string &err) {
    const int n0 = int(nt);
    Cluster *c0 = nullptr, *c1 = nullptr;
    int *nearest = nullptr, *counter = nullptr, *num_sel = nullptr;
    char *keep = nullptr;
    void *tmp = nullptr;
    size_t tmp_bytes = 0;
    int rc = 0;
    do {
        if (!dev_alloc(&c0, sizeof(Cluster) * n0, err) || !dev_alloc(&c1, sizeof(Cluster) * n0, err) ||
            !dev_alloc(&nearest, sizeof(int) * n0, err) || !dev_alloc(&counter, sizeof(int) * 2, err) ||
            !dev_alloc(&num_sel, sizeof(int) * 2, err) || !dev_alloc(&keep, size_t(n0), err)) {
            rc = 3;
            break;
        }
        cub::DeviceSelect::Flagged(nullptr, tmp_bytes, c0, keep, c1, num_sel, n0, st);
        if (!dev_alloc(&tmp, tmp_bytes, err)) {
            rc = 3;
            break;
        }
        cudaMemsetAsync(counter, 0, sizeof(int), st);
        k_ploc_init<<<blocks_for(nt, 256), 256, 0, st>>>(nt, ids2, lo, hi, c0);
        note_launches(1);
        int n = n0;
        int iterations = 0;
        while (n > 1 && iterations < 100000) {
            k_ploc_nearest<<<blocks_for(n, 256), 256, 0, st>>>(n, c0, nearest);
            k_ploc_merge<<<blocks_for(n, 256), 256, 0, st>>>(n, nearest, c0, keep, s.nodes, counter, n0 - 1, par_i,
                                                             par_l);
            if (cub::DeviceSelect::Flagged(tmp, tmp_bytes, c0, keep, c1, num_sel, n, st) != cudaSuccess) {
                err = "PLOC compaction failed";
                rc = 2;
                break;
            }
            note_launches(3);
            int h = 0;
            if (cudaMemcpyAsync(&h, num_sel, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                cudaStreamSynchronize(st) != cudaSuccess) {
                err = "PLOC iteration failed";
                rc = 2;
                break;
            }
            if (h >= n) {  // no pair merged: impossible for a correct nearest search; stop safely
                err = "PLOC made no progress";
                rc = 2;
                break;
            }
            std::swap(c0, c1);
            n = h;
            ++iterations;
        }
        if (rc) break;
        k_leaf_depth<<<blocks_for(nt, 256), 256, 0, st>>>(nt, par_i, par_l, depth + 1);
        note_launches(1);
    } while (false);
    cudaStreamSynchronize(st);
    cudaFree(c0);
    cudaFree(c1);
    cudaFree(nearest);
    cudaFree(counter);
    cudaFree(num_sel);
    cudaFree(keep);
    cudaFree(tmp);
    return rc;
}

// The reachable nodes renumbered in depth-first order from the root (each node's first
// child follows it in memory, so a descent reads neighbouring nodes), the nodes inside
// collapsed leaves dropped: the node array shrinks to the reachable nodes. On the host:
// one download and one upload of the node array.
static int renumber_depth_first(SceneDev &s, cudaStream_t st, std::string &err) {
    const int64_t n = s.node_count;
    if (n < 2) return 0;
    std::vector<DNode> h(static_cast<size_t>(n));
    if (cudaMemcpyAsync(h.data(), s.nodes, sizeof(DNode) * h.size(), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
        err = "BVH layout: node download failed";
        return 2;
    }
    std::vector<int32_t> newid(static_cast<size_t>(n), -1), order, stack{0};
    order.reserve(size_t(n));
    while (!stack.empty()) {
        const int32_t i = stack.back();
        stack.pop_back();
        if (i >= n || newid[i] >= 0 || int64_t(order.size()) >= n) {
            err = "BVH layout: the tree is not a tree";
            return 2;
        }
        newid[i] = int32_t(order.size());
        order.push_back(i);
        if (h[i].d.y >= 0) stack.push_back(h[i].d.y);
        if (h[i].d.x >= 0) stack.push_back(h[i].d.x);
    }
    std::vector<DNode> out(order.size());
    for (size_t k = 0; k < order.size(); ++k) {
        DNode d = h[order[k]];
        if (d.d.x >= 0) d.d.x = newid[d.d.x];
        if (d.d.y >= 0) d.d.y = newid[d.d.y];
        out[k] = d;
    }
    DNode *compact = nullptr;  // the array shrinks to the reachable nodes
    if (!dev_alloc(&compact, sizeof(DNode) * out.size(), err)) return 3;
    if (cudaMemcpyAsync(compact, out.data(), sizeof(DNode) * out.size(), cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
        cudaFree(compact);
        err = "BVH layout: node upload failed";
        return 2;
    }
    cudaFree(s.nodes);
    s.nodes = compact;
    s.node_count = int64_t(out.size());
    return 0;
}

// Builds tris/nodes for `scene` from device vertex/index arrays. Returns 0, 2 (CUDA
// error), 3 (out of memory) or 4 (too many triangles).
int bvh_build(SceneDev &s, const float *d_v, int64_t nv, const int32_t *d_idx, int64_t nt, cudaStream_t st,
              std::string &err) {
    (void)nv;
    if (nt >= (int64_t(1) << 28)) {  // a leaf reference holds the slot in 28 bits
        err = "scenes are limited to 2^28 - 1 triangles";
        return 4;
    }
    s.tri_count = nt;
    const int64_t n_nodes = nt >= 2 ? nt - 1 : 1;
    s.node_count = n_nodes;
    if (!dev_alloc(&s.tris, sizeof(DTri) * (size_t)std::max<int64_t>(nt, 1), err)) return 3;
    if (!dev_alloc(&s.nodes, sizeof(DNode) * (size_t)n_nodes, err)) return 3;
    if (nt < 2) {
        // 0 or 1 triangle: one root whose two children are both slot 0. With no triangle,
        // slot 0 is all zeros (zero determinant: never hit). A second visit of the only
        // triangle is harmless. (An inverted box is not empty under the min/max slab test.)
        if (cudaMemsetAsync(s.tris, 0, sizeof(DTri), st) != cudaSuccess) return 2;
        DNode root;
        const float inf = std::numeric_limits<float>::infinity();
        root.a = make_float4(inf, -inf, inf, -inf);
        root.b = make_float4(inf, -inf, inf, -inf);
        root.c = make_float4(inf, -inf, inf, -inf);
        root.d = make_int4(-1, -1, 0, 0);  // ~0 = slot 0
        if (nt == 1) {
            float hv[9];
            int32_t hi[3];
            if (cudaMemcpyAsync(hi, d_idx, sizeof(hi), cudaMemcpyDeviceToHost, st) != cudaSuccess) return 2;
            cudaStreamSynchronize(st);
            for (int k = 0; k < 3; ++k)
                if (cudaMemcpyAsync(hv + 3 * k, d_v + 3 * (int64_t)hi[k], 3 * sizeof(float), cudaMemcpyDeviceToHost,
                                    st) != cudaSuccess)
                    return 2;
            cudaStreamSynchronize(st);
            float lo[3], hiB[3];
            for (int a = 0; a < 3; ++a) {
                float mn = std::min(hv[a], std::min(hv[3 + a], hv[6 + a]));
                float mx = std::max(hv[a], std::max(hv[3 + a], hv[6 + a]));
                float pad = std::max(std::fabs(mn), std::fabs(mx)) * 4e-6f + 1e-6f;
                lo[a] = mn - pad;
                hiB[a] = mx + pad;
            }
            root.a = make_float4(lo[0], hiB[0], lo[1], hiB[1]);
            root.c.x = lo[2];
            root.c.y = hiB[2];
            DTri T;
            T.v0 = make_float4(hv[0], hv[1], hv[2], 0.f);  // bit pattern of int 0
            T.e1 = make_float4(hv[3] - hv[0], hv[4] - hv[1], hv[5] - hv[2], 0.f);
            T.e2 = make_float4(hv[6] - hv[0], hv[7] - hv[1], hv[8] - hv[2], 0.f);
            if (cudaMemcpyAsync(s.tris, &T, sizeof(T), cudaMemcpyHostToDevice, st) != cudaSuccess) return 2;
        }
        if (cudaMemcpyAsync(s.nodes, &root, sizeof(root), cudaMemcpyHostToDevice, st) != cudaSuccess) return 2;
        cudaStreamSynchronize(st);
        s.max_depth = nt == 1 ? 1 : 0;
        s.leaf_count = nt;
        return 0;
    }

    float *lo = nullptr, *hi = nullptr;
    unsigned *cb = nullptr;
    uint64_t *keys = nullptr, *keys2 = nullptr;
    int32_t *ids = nullptr, *ids2 = nullptr, *par_i = nullptr, *par_l = nullptr;
    int *counters = nullptr, *depth = nullptr;
    void *tmp = nullptr;
    size_t tmp_bytes = 0;
    int rc = 0;
    auto fail = [&](int code) {
        rc = code;
        return code;
    };
    do {
        if (!dev_alloc(&lo, sizeof(float) * 3 * nt, err) || !dev_alloc(&hi, sizeof(float) * 3 * nt, err) ||
            !dev_alloc(&cb, sizeof(unsigned) * 6, err) || !dev_alloc(&keys, sizeof(uint64_t) * nt, err) ||
            !dev_alloc(&keys2, sizeof(uint64_t) * nt, err) || !dev_alloc(&ids, sizeof(int32_t) * nt, err) ||
            !dev_alloc(&ids2, sizeof(int32_t) * nt, err) || !dev_alloc(&par_i, sizeof(int32_t) * n_nodes, err) ||
            !dev_alloc(&par_l, sizeof(int32_t) * nt, err) || !dev_alloc(&counters, sizeof(int) * n_nodes, err) ||
            !dev_alloc(&depth, sizeof(int) * 2, err)) {
            fail(3);
            break;
        }
        unsigned init[6] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u};
        cudaMemcpyAsync(cb, init, sizeof(init), cudaMemcpyHostToDevice, st);
        cudaMemsetAsync(counters, 0, sizeof(int) * n_nodes, st);
        cudaMemsetAsync(depth, 0, sizeof(int) * 2, st);
        cudaMemsetAsync(par_i, 0xff, sizeof(int32_t) * n_nodes, st);  // root keeps -1
        const int T = 256;
        k_bounds<<<blocks_for(nt, T), T, 0, st>>>(d_v, d_idx, nt, lo, hi, cb);
        k_morton<<<blocks_for(nt, T), T, 0, st>>>(lo, hi, nt, cb, keys, ids);
        note_launches(2);
        if (cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, keys, keys2, ids, ids2, (int)nt, 0, 63, st) !=
            cudaSuccess) {
            err = "radix sort size query failed";
            fail(2);
            break;
        }
        if (!dev_alloc(&tmp, tmp_bytes, err)) {
            fail(3);
            break;
        }
        if (cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, keys, keys2, ids, ids2, (int)nt, 0, 63, st) !=
            cudaSuccess) {
            err = "radix sort failed";
            fail(2);
            break;
        }
        k_write_tris<<<blocks_for(nt, T), T, 0, st>>>(d_v, d_idx, ids2, nt, s.tris);
        if (g_bvh_builder == 0) {
            note_launches(1);
            const int prc = build_ploc(s, nt, ids2, lo, hi, par_i, par_l, depth, st, err);
            if (prc) {
                fail(prc);
                break;
            }
        } else {
            k_karras<<<blocks_for(nt - 1, T), T, 0, st>>>(keys2, nt, s.nodes, par_i, par_l);
            k_refit<<<blocks_for(nt, T), T, 0, st>>>(nt, ids2, lo, hi, s.nodes, par_i, par_l, counters, depth);
            k_leaf_depth<<<blocks_for(nt, T), T, 0, st>>>(nt, par_i, par_l, depth + 1);
            note_launches(4);
        }
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            err = std::string("BVH build: ") + cudaGetErrorString(e);
            fail(2);
            break;
        }
        const int orc = optimize_tree(s, nt, par_i, par_l, st, err);
        if (orc) {
            fail(orc);
            break;
        }
        if (g_bvh_optimize > 0) {  // the depth of the tree as it now is
            cudaMemsetAsync(depth + 1, 0, sizeof(int), st);
            k_leaf_depth<<<blocks_for(nt, T), T, 0, st>>>(nt, par_i, par_l, depth + 1);
            note_launches(1);
        }
        const int lrc = collapse_leaves(s, nt, par_i, par_l, counters, st, err);
        if (lrc) {
            fail(lrc);
            break;
        }
        const int drc = renumber_depth_first(s, st, err);
        if (drc) {
            fail(drc);
            break;
        }
        int hd[2];
        cudaMemcpy(hd, depth, sizeof(hd), cudaMemcpyDeviceToHost);
        s.max_depth = hd[1];
        s.leaf_count = nt;
    } while (false);
    cudaFree(lo);
    cudaFree(hi);
    cudaFree(cb);
    cudaFree(keys);
    cudaFree(keys2);
    cudaFree(ids);
    cudaFree(ids2);
    cudaFree(par_i);
    cudaFree(par_l);
    cudaFree(counters);
    cudaFree(depth);
    cudaFree(tmp);
    return rc;
}

namespace {

// Triangle records of new vertex positions: slot s keeps its triangle (the original id in
// v0.w), as k_write_tris forms them.
__global__ void k_refit_tris(int64_t nt, const float *__restrict__ v, const int32_t *__restrict__ idx,
                             DTri *__restrict__ tris) {
    const int64_t s = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (s >= nt) return;
    const float idbits = tris[s].v0.w;
    const int64_t t = __float_as_int(idbits);
    const float *p0 = v + 3 * int64_t(idx[3 * t + 0]);
    const float *p1 = v + 3 * int64_t(idx[3 * t + 1]);
    const float *p2 = v + 3 * int64_t(idx[3 * t + 2]);
    DTri T;
    T.v0 = make_float4(p0[0], p0[1], p0[2], idbits);
    T.e1 = make_float4(p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2], 0.f);
    T.e2 = make_float4(p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2], 0.f);
    tris[s] = T;
}

// One level of the bottom-up refit: each node's two child boxes from its children (a
// leaf: the padded boxes of its triangles, as k_bounds pads them; a node: the union of
// its own two boxes, refitted one level deeper).
__global__ void k_refit_level(int64_t count, const int32_t *__restrict__ order, DNode *nodes,
                              const DTri *__restrict__ tris, const float *__restrict__ v,
                              const int32_t *__restrict__ idx) {
    const int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (k >= count) return;
    const int i = order[k];
    const int c[2] = {nodes[i].d.x, nodes[i].d.y};
    Box bx[2];
    for (int w = 0; w < 2; ++w) {
        for (int a = 0; a < 3; ++a) {
            bx[w].lo[a] = __int_as_float(0x7f800000);
            bx[w].hi[a] = -__int_as_float(0x7f800000);
        }
        if (c[w] < 0) {
            const int ref = ~c[w];
            for (int slot = ref >> 3; slot <= (ref >> 3) + (ref & 7); ++slot) {
                const int64_t t = __float_as_int(tris[slot].v0.w);
                for (int a = 0; a < 3; ++a) {
                    const float x0 = v[3 * int64_t(idx[3 * t + 0]) + a];
                    const float x1 = v[3 * int64_t(idx[3 * t + 1]) + a];
                    const float x2 = v[3 * int64_t(idx[3 * t + 2]) + a];
                    const float mn = fminf(x0, fminf(x1, x2)), mx = fmaxf(x0, fmaxf(x1, x2));
                    const float pad = fmaxf(fabsf(mn), fabsf(mx)) * 4e-6f + 1e-6f;
                    bx[w].lo[a] = fminf(bx[w].lo[a], mn - pad);
                    bx[w].hi[a] = fmaxf(bx[w].hi[a], mx + pad);
                }
            }
        } else {
            const DNode cn = nodes[c[w]];
            const Box b0 = child_box(cn, 0), b1 = child_box(cn, 1);
            for (int a = 0; a < 3; ++a) {
                bx[w].lo[a] = fminf(b0.lo[a], b1.lo[a]);
                bx[w].hi[a] = fmaxf(b0.hi[a], b1.hi[a]);
            }
        }
    }
    DNode &n = nodes[i];
    n.a = make_float4(bx[0].lo[0], bx[0].hi[0], bx[0].lo[1], bx[0].hi[1]);
    n.b = make_float4(bx[1].lo[0], bx[1].hi[0], bx[1].lo[1], bx[1].hi[1]);
    n.c = make_float4(bx[0].lo[2], bx[0].hi[2], bx[1].lo[2], bx[1].hi[2]);
}

}  // namespace

int bvh_refit(SceneDev &s, const float *d_v, cudaStream_t st, std::string &err) {
    const int64_t nt = s.tri_count;
    if (nt < 2) {  // the one-node tree of 0 or 1 triangle: built again
        cudaFree(s.tris);
        cudaFree(s.nodes);
        s.tris = nullptr;
        s.nodes = nullptr;
        return bvh_build(s, d_v, s.vertex_count, s.indices, nt, st, err);
    }
    if (!s.refit_order) {
        // the reachable internal nodes, level by level from the root (host breadth-first
        // walk over the child references)
        std::vector<DNode> h(size_t(s.node_count));
        if (cudaMemcpy(h.data(), s.nodes, sizeof(DNode) * h.size(), cudaMemcpyDeviceToHost) != cudaSuccess) {
            err = "refit: node download failed";
            return 2;
        }
        std::vector<int32_t> order{0}, next;
        std::vector<int64_t> levels{0};
        size_t begin = 0;
        while (begin < order.size()) {
            const size_t end = order.size();
            for (size_t k = begin; k < end; ++k)
                for (int c : {h[order[k]].d.x, h[order[k]].d.y})
                    if (c >= 0) order.push_back(c);
            levels.push_back(int64_t(end));
            begin = end;
        }
        if (!dev_alloc(&s.refit_order, sizeof(int32_t) * order.size(), err)) return 3;
        if (cudaMemcpy(s.refit_order, order.data(), sizeof(int32_t) * order.size(), cudaMemcpyHostToDevice) !=
            cudaSuccess) {
            err = "refit: order upload failed";
            return 2;
        }
        s.refit_levels = levels;
    }
    const int T = 256;
    k_refit_tris<<<blocks_for(nt, T), T, 0, st>>>(nt, d_v, s.indices, s.tris);
    note_launches(1);
    for (size_t l = s.refit_levels.size() - 1; l-- > 0;) {  // deepest level first
        const int64_t b = s.refit_levels[l], e = s.refit_levels[l + 1];
        k_refit_level<<<blocks_for(e - b, T), T, 0, st>>>(e - b, s.refit_order + b, s.nodes, s.tris, d_v, s.indices);
        note_launches(1);
    }
    const cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        err = std::string("BVH refit: ") + cudaGetErrorString(e);
        return 2;
    }
    return 0;
}

}  // namespace hsr
