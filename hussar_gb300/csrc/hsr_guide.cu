// GuidingWrapper::step (libhussar/include/hussar/integrators/path.h:119-126) on the
// device, one thread per pose (trees have at most 2048 nodes):
//   build   leaf energy = sqrt(sum w d^2 * leaf area) (second moment, path.h:232),
//           internal energy = sum of its children, first-child probability = share;
//   copy    sampling tree := built training tree;
//   refine  new training topology: a subtree whose energy fraction is at most the split
//           threshold (0.005, path.h:230) collapses to a leaf; a leaf above it splits in
//           halves (recursively, each half taking half the fraction); statistics reset.
#include "hsr_guide.cuh"
#include "hsr_internal.h"

namespace hsr {

namespace {

__global__ void k_guide_reset(int P, int *samp_child, float *samp_p, int *train_child, float *train_acc,
                              int *train_count) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    samp_child[size_t(p) * kGuideMaxNodes] = -1;
    samp_p[size_t(p) * kGuideMaxNodes] = 0.5f;
    train_child[size_t(p) * kGuideMaxNodes] = -1;
    float *acc = train_acc + size_t(p) * kGuideMaxNodes * 3;
    acc[0] = acc[1] = acc[2] = 0.f;
    train_count[p] = 1;
}

__global__ void k_guide_step(int P, const int *__restrict__ active, int *samp_child, float *samp_p, int *train_child,
                             float *train_acc, int *train_count, float *scratch_e, int *scratch_i) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P || !active[p]) return;
    const size_t base = size_t(p) * kGuideMaxNodes;
    int *tc = train_child + base;
    float *acc = train_acc + base * 3;
    int *sc = samp_child + base;
    float *sp = samp_p + base;
    float *e = scratch_e + base;
    int *depth = scratch_i + 2 * base;
    int *nchild = scratch_i + 2 * base + kGuideMaxNodes;
    const int count = min(max(train_count[p], 1), kGuideMaxNodes);

    // depths (children always follow their parent)
    depth[0] = 0;
    for (int i = 0; i < count; ++i) {
        const int c = tc[i];
        if (c >= 0 && c + 1 < count) depth[c] = depth[c + 1] = depth[i] + 1;
    }
    // build: energies bottom-up
    for (int i = count - 1; i >= 0; --i) {
        const int c = tc[i];
        if (c < 0) {
            const float area = ldexpf(1.f, -depth[i]);
            e[i] = sqrtf(fmaxf(acc[3 * i + 2], 0.f) * area);
        } else {
            e[i] = e[c] + e[c + 1];
        }
    }
    // copy to the sampling tree
    for (int i = 0; i < count; ++i) {
        const int c = tc[i];
        sc[i] = c;
        if (c >= 0) {
            const float s = e[c] + e[c + 1];
            sp[i] = s > 0.f ? e[c] / s : 0.5f;
        } else {
            sp[i] = 0.5f;
        }
    }
    // refine into a new training topology
    const float total = e[0];
    int ncount = 1;
    if (total > 0.f) {
        struct Item {
            int old;
            float f;
            int d;
            int ni;
        } stack[2 * kGuideMaxDepth + 4];
        int top = 0;
        stack[top++] = Item{0, 1.f, 0, 0};
        while (top > 0) {
            const Item it = stack[--top];
            const bool internal = it.old >= 0 && tc[it.old] >= 0;
            const bool split = it.f > kGuideSplitThreshold && it.d < kGuideMaxDepth &&
                               ncount + 2 <= kGuideMaxNodes && top + 2 <= 2 * kGuideMaxDepth + 4;
            if (!split) {
                nchild[it.ni] = -1;
                continue;
            }
            const int c = ncount;
            ncount += 2;
            nchild[it.ni] = c;
            if (internal) {
                const int oc = tc[it.old];
                const float eo = e[it.old];
                const float f0 = eo > 0.f ? it.f * (e[oc] / eo) : 0.5f * it.f;
                const float f1 = eo > 0.f ? it.f * (e[oc + 1] / eo) : 0.5f * it.f;
                stack[top++] = Item{oc + 1, f1, it.d + 1, c + 1};
                stack[top++] = Item{oc, f0, it.d + 1, c};
            } else {
                stack[top++] = Item{-1, 0.5f * it.f, it.d + 1, c + 1};
                stack[top++] = Item{-1, 0.5f * it.f, it.d + 1, c};
            }
        }
        for (int i = 0; i < ncount; ++i) tc[i] = nchild[i];
    } else {
        ncount = count;  // no information: keep the topology
    }
    for (int i = 0; i < 3 * ncount; ++i) acc[i] = 0.f;
    train_count[p] = ncount;
}

}  // namespace

size_t guide_bytes_per_pose() {
    // samp child + p, train child + 3 acc, scratch energy + depth + new child, count
    return size_t(kGuideMaxNodes) * (4 + 4 + 4 + 12 + 4 + 8) + 16;
}

int launch_guide_reset(int P, int *samp_child, float *samp_p, int *train_child, float *train_acc, int *train_count,
                       cudaStream_t st) {
    k_guide_reset<<<(P + 127) / 128, 128, 0, st>>>(P, samp_child, samp_p, train_child, train_acc, train_count);
    note_launches(1);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

int launch_guide_step(int P, const int *active, int *samp_child, float *samp_p, int *train_child, float *train_acc,
                      int *train_count, float *scratch_e, int *scratch_i, cudaStream_t st) {
    k_guide_step<<<(P + 63) / 64, 64, 0, st>>>(P, active, samp_child, samp_p, train_child, train_acc, train_count,
                                               scratch_e, scratch_i);
    note_launches(1);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

}  // namespace hsr
