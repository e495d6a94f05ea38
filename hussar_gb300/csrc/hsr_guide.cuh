// Path guiding of the TX primary sample square on the device: a 2-D adaptive binary
// tree (regions halved at their midpoint, axis alternating with depth) mixed with a
// uniform density, the role libguiding's BTree plays behind GuidingWrapper
// (libhussar/include/hussar/integrators/path.h:17-131, settings path.h:229-232:
// uniformProb 0.1, splitThreshold 0.005, secondMoment).
//
// Per pose, two trees live in device memory:
//   sampling: child index (-1 = leaf) and the probability of the first child
//   training: child index and per-leaf accumulators [3]; the step reads the second
//             moment sum w d^2 (slot 2), the only statistic the tree is built from
// A step (k_guide_step) builds the training tree's energies from its accumulators,
// copies it into the sampling tree and refines the training tree (split leaves above
// the threshold fraction, collapse subtrees below it), as GuidingWrapper::step does
// (path.h:119-126).
#pragma once
#include "hsr_common.cuh"
#include "hsr_internal.h"

namespace hsr {

constexpr int kGuideMaxDepth = 24;
constexpr float kGuideUniformProb = 0.1f;    // path.h:229
constexpr float kGuideSplitThreshold = 0.005f;  // path.h:230

struct GuideView {  // device pointers for one batch, [pose][kGuideMaxNodes]
    const int *samp_child;
    const float *samp_pfirst;
    const int *train_child;
    float *train_acc;  // [pose][node][3]
};

// The tree helpers read through plain pointers: global memory, or a CTA's shared-memory
// copy of the pose's trees (the wavefront kernel stages them when it switches pose).

// Tree density of the sampling tree at x (relative to uniform); descends by position.
__device__ __forceinline__ float guide_tree_pdf(const int *child, const float *pfirst, float x0, float x1) {
    float pdf = 1.f;
    int node = 0;
    float lo0 = 0.f, lo1 = 0.f, s0 = 1.f, s1 = 1.f;
    int depth = 0;
    while (depth < kGuideMaxDepth) {
        const int c = child[node];
        if (c < 0) break;
        const float p0 = pfirst[node];
        if ((depth & 1) == 0) {
            s0 *= 0.5f;
            if (x0 < lo0 + s0) {
                pdf *= 2.f * p0;
                node = c;
            } else {
                pdf *= 2.f * (1.f - p0);
                lo0 += s0;
                node = c + 1;
            }
        } else {
            s1 *= 0.5f;
            if (x1 < lo1 + s1) {
                pdf *= 2.f * p0;
                node = c;
            } else {
                pdf *= 2.f * (1.f - p0);
                lo1 += s1;
                node = c + 1;
            }
        }
        ++depth;
    }
    return pdf;
}

// Warps x (local coordinates of the unit square) through the sampling tree; returns the
// tree density at the warped point.
__device__ __forceinline__ float guide_tree_sample(const int *child, const float *pfirst, float &x0, float &x1) {
    float pdf = 1.f;
    int node = 0;
    float lo0 = 0.f, lo1 = 0.f, s0 = 1.f, s1 = 1.f;
    int depth = 0;
    while (depth < kGuideMaxDepth) {
        const int c = child[node];
        if (c < 0) break;
        const float p0 = pfirst[node];
        float &x = (depth & 1) == 0 ? x0 : x1;
        if (x < p0) {
            x = p0 > 0.f ? x / p0 : 0.f;
            pdf *= 2.f * p0;
            node = c;
            if ((depth & 1) == 0)
                s0 *= 0.5f;
            else
                s1 *= 0.5f;
        } else {
            x = p0 < 1.f ? (x - p0) / (1.f - p0) : 0.f;
            pdf *= 2.f * (1.f - p0);
            node = c + 1;
            if ((depth & 1) == 0) {
                s0 *= 0.5f;
                lo0 += s0;
            } else {
                s1 *= 0.5f;
                lo1 += s1;
            }
        }
        x = fminf(fmaxf(x, 0.f), 0.99999994f);
        ++depth;
    }
    x0 = fminf(lo0 + x0 * s0, 0.99999994f);
    x1 = fminf(lo1 + x1 * s1, 0.99999994f);
    return pdf;
}

// GuidingWrapper::sample (path.h:54-82): mixture of uniform (probability 0.1) and tree.
// Warps (x0, x1) in place and returns the mixture pdf.
__device__ __forceinline__ float guide_sample(const int *child, const float *pfirst, float &x0, float &x1) {
    const float u = kGuideUniformProb;
    float pdf = 1.f - u;
    if (x0 < u) {
        x0 /= u;
        pdf *= guide_tree_pdf(child, pfirst, x0, x1);
    } else {
        x0 -= u;
        x0 /= 1.f - u;
        pdf *= guide_tree_sample(child, pfirst, x0, x1);
    }
    return pdf + u;
}

// The training tree's leaf at x (GuidingWrapper::splat's lookup, path.h:96-111).
__device__ __forceinline__ int guide_leaf(const int *child, float x0, float x1) {
    int node = 0;
    float lo0 = 0.f, lo1 = 0.f, s0 = 1.f, s1 = 1.f;
    int depth = 0;
    while (depth < kGuideMaxDepth) {
        const int c = child[node];
        if (c < 0) break;
        if ((depth & 1) == 0) {
            s0 *= 0.5f;
            if (x0 < lo0 + s0) {
                node = c;
            } else {
                lo0 += s0;
                node = c + 1;
            }
        } else {
            s1 *= 0.5f;
            if (x1 < lo1 + s1) {
                node = c;
            } else {
                lo1 += s1;
                node = c + 1;
            }
        }
        ++depth;
    }
    return node;
}

}  // namespace hsr
