// CPU check of the device traversal code, compiled from the product's own header
// (hussar_gb300/csrc/hsr_traverse.cuh) with host definitions of the CUDA intrinsics
// (host_shim.h): a binary tree in the kernels' DNode layout (median split, leaves of up to
// argv[2] triangles in consecutive slots, boxes padded like the device build) answers
// every ray through
// hsr::closest_hit / hsr::any_hit, and brute force over all triangles with the same
// triangle test and tie rule answers it again.
//
// Input (binary, little endian): int64 nv, nt, nr; float v[nv][3]; int32 idx[nt][3];
// float o[nr][3], d[nr][3], tfar[nr]. Output: one line
// "depth D closest_mismatch C any_mismatch A stack_status S nodes_per_ray X".
#include "host_shim.h"
#include "hsr_traverse.cuh"

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

using namespace hsr;

struct Item {
    float lo[3], hi[3], c[3];
    int slot;
};

static void box_of(const std::vector<Item> &it, int a, int b, float *lo, float *hi) {
    for (int k = 0; k < 3; ++k) {
        lo[k] = it[a].lo[k];
        hi[k] = it[a].hi[k];
    }
    for (int i = a + 1; i < b; ++i)
        for (int k = 0; k < 3; ++k) {
            lo[k] = std::min(lo[k], it[i].lo[k]);
            hi[k] = std::max(hi[k], it[i].hi[k]);
        }
}

// Median split over centroids; returns the child reference of range [a, b). A range of at
// most `leaf` triangles (not the root's) becomes a leaf: its records are appended to
// `out` and referenced as ~((first slot << 3) | (count - 1)).
static int build(std::vector<Item> &it, int a, int b, std::vector<DNode> &nodes, int depth, int &max_depth,
                 int leaf, const std::vector<DTri> &tris, std::vector<DTri> &out) {
    max_depth = std::max(max_depth, depth);
    if (b - a <= leaf && depth > 0) {
        const int first = int(out.size());
        for (int i = a; i < b; ++i) out.push_back(tris[it[i].slot]);
        return ~((first << 3) | (b - a - 1));
    }
    const int id = int(nodes.size());
    nodes.emplace_back();
    float clo[3] = {1e30f, 1e30f, 1e30f}, chi[3] = {-1e30f, -1e30f, -1e30f};
    for (int i = a; i < b; ++i)
        for (int k = 0; k < 3; ++k) {
            clo[k] = std::min(clo[k], it[i].c[k]);
            chi[k] = std::max(chi[k], it[i].c[k]);
        }
    int ax = 0;
    for (int k = 1; k < 3; ++k)
        if (chi[k] - clo[k] > chi[ax] - clo[ax]) ax = k;
    const int mid = (a + b) / 2;
    std::nth_element(it.begin() + a, it.begin() + mid, it.begin() + b,
                     [ax](const Item &x, const Item &y) { return x.c[ax] < y.c[ax]; });
    float l0[3], h0[3], l1[3], h1[3];
    box_of(it, a, mid, l0, h0);
    box_of(it, mid, b, l1, h1);
    const int c0 = build(it, a, mid, nodes, depth + 1, max_depth, leaf, tris, out);
    const int c1 = build(it, mid, b, nodes, depth + 1, max_depth, leaf, tris, out);
    DNode &n = nodes[id];
    n.a = make_float4(l0[0], h0[0], l0[1], h0[1]);
    n.b = make_float4(l1[0], h1[0], l1[1], h1[1]);
    n.c = make_float4(l0[2], h0[2], l1[2], h1[2]);
    n.d = make_int4(c0, c1, 0, 0);
    return id;
}

int main(int argc, char **argv) {
    if (argc < 2) return 2;
    const int leaf = argc > 2 ? std::atoi(argv[2]) : 1;
    if (leaf < 1 || leaf > 8) return 2;
    FILE *f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    int64_t hdr[3];
    if (std::fread(hdr, 8, 3, f) != 3) return 2;
    const int64_t nv = hdr[0], nt = hdr[1], nr = hdr[2];
    std::vector<float> v(3 * nv), o(3 * nr), d(3 * nr), tf(nr);
    std::vector<int32_t> idx(3 * nt);
    if (std::fread(v.data(), 4, v.size(), f) != v.size() || std::fread(idx.data(), 4, idx.size(), f) != idx.size() ||
        std::fread(o.data(), 4, o.size(), f) != o.size() || std::fread(d.data(), 4, d.size(), f) != d.size() ||
        std::fread(tf.data(), 4, tf.size(), f) != tf.size())
        return 2;
    std::fclose(f);
    if (nt < 2) return 2;
    std::vector<DTri> tris(nt);
    std::vector<Item> items(nt);
    for (int64_t t = 0; t < nt; ++t) {
        const float *p[3] = {&v[3 * idx[3 * t]], &v[3 * idx[3 * t + 1]], &v[3 * idx[3 * t + 2]]};
        tris[t].v0 = make_float4(p[0][0], p[0][1], p[0][2], __int_as_float(int(t)));
        tris[t].e1 = make_float4(p[1][0] - p[0][0], p[1][1] - p[0][1], p[1][2] - p[0][2], 0.f);
        tris[t].e2 = make_float4(p[2][0] - p[0][0], p[2][1] - p[0][1], p[2][2] - p[0][2], 0.f);
        for (int a = 0; a < 3; ++a) {
            const float mn = std::min(p[0][a], std::min(p[1][a], p[2][a]));
            const float mx = std::max(p[0][a], std::max(p[1][a], p[2][a]));
            const float pad = std::max(std::fabs(mn), std::fabs(mx)) * 4e-6f + 1e-6f;
            items[t].lo[a] = mn - pad;
            items[t].hi[a] = mx + pad;
            items[t].c[a] = 0.5f * mn + 0.5f * mx;
        }
        items[t].slot = int(t);
    }
    std::vector<DNode> nodes;
    nodes.reserve(nt);
    std::vector<DTri> leaf_tris;
    leaf_tris.reserve(nt);
    int depth = 0;
    build(items, 0, int(nt), nodes, 0, depth, leaf, tris, leaf_tris);
    unsigned status = 0;
    int64_t bad_c = 0, bad_a = 0;
    TraversalCounters cnt{0u, 0u};
    for (int64_t r = 0; r < nr; ++r) {
        const f3 oo = mk3(o[3 * r], o[3 * r + 1], o[3 * r + 2]);
        const f3 dd = mk3(d[3 * r], d[3 * r + 1], d[3 * r + 2]);
        float tb;
        int pb;
        const int slot =
            closest_hit<true>(nodes.data(), leaf_tris.data(), oo, dd, kEpsilon, INFINITY, tb, pb, &status, &cnt);
        float bt = INFINITY;
        int bp = 0x7fffffff;
        for (int64_t t = 0; t < nt; ++t) {
            float th;
            if (tri_test(tris[t], oo, dd, kEpsilon, INFINITY, th) && (th < bt || (th == bt && int(t) < bp))) {
                bt = th;
                bp = int(t);
            }
        }
        const int gp = slot < 0 ? 0x7fffffff : __float_as_int(leaf_tris[slot].v0.w);
        if (gp != bp || (slot >= 0 && __float_as_uint(tb) != __float_as_uint(bt))) ++bad_c;
        bool occ = false;
        for (int64_t t = 0; t < nt && !occ; ++t) {
            float th;
            occ = tri_test(tris[t], oo, dd, kEpsilon, tf[r], th);
        }
        if (any_hit<false>(nodes.data(), leaf_tris.data(), oo, dd, kEpsilon, tf[r], &status, nullptr) != occ) ++bad_a;
    }
    std::printf("depth %d closest_mismatch %lld any_mismatch %lld stack_status %u nodes_per_ray %.2f "
                "tris_per_ray %.2f\n",
                depth, (long long)bad_c, (long long)bad_a, status, double(cnt.nodes) / double(nr),
                double(cnt.tris) / double(nr));
    return 0;
}
