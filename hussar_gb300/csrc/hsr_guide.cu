// GuidingWrapper::step (libhussar/include/hussar/integrators/path.h:119-126) on the
// device, one CTA per pose with the tree staged in shared memory (at most 2048 nodes;
// the order-dependent passes run on one thread, the copies on all):
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

__global__ void __launch_bounds__(256) k_guide_step(const int *__restrict__ active, int *samp_child, float *samp_p,
                                                    int *train_child, float *train_acc, int *train_count) {
    const int p = blockIdx.x;
    if (!active[p]) return;  // uniform over the CTA
    __shared__ int tc_s[kGuideMaxNodes];    // training topology
    __shared__ float m2_s[kGuideMaxNodes];  // second-moment statistic of each node
    __shared__ float e_s[kGuideMaxNodes];   // energies
    __shared__ int aux_s[kGuideMaxNodes];   // depths, then the new topology
    __shared__ int s_ncount;
    const size_t base = size_t(p) * kGuideMaxNodes;
    int *tc = train_child + base;
    float *acc = train_acc + base * 3;
    int *sc = samp_child + base;
    float *sp = samp_p + base;
    const int count = min(max(train_count[p], 1), kGuideMaxNodes);
    for (int i = threadIdx.x; i < count; i += blockDim.x) {
        tc_s[i] = tc[i];
        m2_s[i] = acc[3 * i + 2];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        // depths (children always follow their parent), then energies bottom-up
        aux_s[0] = 0;
        for (int i = 0; i < count; ++i) {
            const int c = tc_s[i];
            if (c >= 0 && c + 1 < count) aux_s[c] = aux_s[c + 1] = aux_s[i] + 1;
        }
        for (int i = count - 1; i >= 0; --i) {
            const int c = tc_s[i];
            if (c < 0) {
                const float area = ldexpf(1.f, -aux_s[i]);
                e_s[i] = sqrtf(fmaxf(m2_s[i], 0.f) * area);
            } else {
                e_s[i] = e_s[c] + e_s[c + 1];
            }
        }
    }
    __syncthreads();
    // copy to the sampling tree
    for (int i = threadIdx.x; i < count; i += blockDim.x) {
        const int c = tc_s[i];
        sc[i] = c;
        if (c >= 0) {
            const float s = e_s[c] + e_s[c + 1];
            sp[i] = s > 0.f ? e_s[c] / s : 0.5f;
        } else {
            sp[i] = 0.5f;
        }
    }
    // refine into a new training topology (aux_s: new child links)
    const float total = e_s[0];
    if (threadIdx.x == 0) {
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
                const bool internal = it.old >= 0 && tc_s[it.old] >= 0;
                const bool split = it.f > kGuideSplitThreshold && it.d < kGuideMaxDepth &&
                                   ncount + 2 <= kGuideMaxNodes && top + 2 <= 2 * kGuideMaxDepth + 4;
                if (!split) {
                    aux_s[it.ni] = -1;
                    continue;
                }
                const int c = ncount;
                ncount += 2;
                aux_s[it.ni] = c;
                if (internal) {
                    const int oc = tc_s[it.old];
                    const float eo = e_s[it.old];
                    const float f0 = eo > 0.f ? it.f * (e_s[oc] / eo) : 0.5f * it.f;
                    const float f1 = eo > 0.f ? it.f * (e_s[oc + 1] / eo) : 0.5f * it.f;
                    stack[top++] = Item{oc + 1, f1, it.d + 1, c + 1};
                    stack[top++] = Item{oc, f0, it.d + 1, c};
                } else {
                    stack[top++] = Item{-1, 0.5f * it.f, it.d + 1, c + 1};
                    stack[top++] = Item{-1, 0.5f * it.f, it.d + 1, c};
                }
            }
        } else {
            ncount = count;  // no information: keep the topology
        }
        s_ncount = ncount;
    }
    __syncthreads();
    const int ncount = s_ncount;
    if (total > 0.f)
        for (int i = threadIdx.x; i < ncount; i += blockDim.x) tc[i] = aux_s[i];
    for (int i = threadIdx.x; i < 3 * ncount; i += blockDim.x) acc[i] = 0.f;
    if (threadIdx.x == 0) train_count[p] = ncount;
}

}  // namespace

size_t guide_bytes_per_pose() {
    // samp child + p, train child + 3 acc, count, and the guided schedule (kGuideMaxIters
    // iterations x 32 B)
    return size_t(kGuideMaxNodes) * (4 + 4 + 4 + 12) + size_t(kGuideMaxIters) * 32 + 16;
}

int launch_guide_reset(int P, int *samp_child, float *samp_p, int *train_child, float *train_acc, int *train_count,
                       cudaStream_t st) {
    k_guide_reset<<<(P + 127) / 128, 128, 0, st>>>(P, samp_child, samp_p, train_child, train_acc, train_count);
    note_launches(1);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

int launch_guide_step(int P, const int *active, int *samp_child, float *samp_p, int *train_child, float *train_acc,
                      int *train_count, cudaStream_t st) {
    k_guide_step<<<P, 256, 0, st>>>(active, samp_child, samp_p, train_child, train_acc, train_count);
    note_launches(1);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

}  // namespace hsr
