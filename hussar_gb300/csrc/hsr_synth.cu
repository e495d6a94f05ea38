// Synthesis of the range spectrum from the fine range histogram (HSR_SPLAT_FINE_SYNTH).
//
// The trace kernels add each next-event contribution c at fractional range bin b into a
// fine histogram with OS = 8 sub-bins per range bin and four moment terms:
//   k = round(8 b) mod K (K = 8 N), eps = b - k/8 (bins), h_d[k] += c eps^d / d! (d < 4).
// The sampled IF chirp of one contribution is c exp(j 2 pi b n / N), n < N; expanding in
// eps to third order, the spectrum (frame row, the reference's Frame layout) is
//   frame[m] = sum_d sum_k h_d[k] g_d(k - 8 m),
//   g_d(j) = (1/N) sum_{n<N} (j 2 pi n / N)^d exp(j 2 pi (j/8) n / N)   (j mod K),
// i.e. the untruncated finite-N Dirichlet kernel and its first three derivatives; the
// reference's Frame::splat<16> (radar.h:564-626) is its large-N limit cut at +-16 bins.
// The Taylor remainder is below (pi/8)^4 / 24 * |c| per contribution (1e-3 at the end
// of the chirp, ~3e-4 averaged over it).
//
// As a real GEMM: C[P x 2N] = A[P x 8K] * B[8K x 2N] with A = [Re h0..h3 | Im h0..h3]
// and B = [[Re G, Im G], [-Im G, Re G]]. On the tensor cores (tcgen05.mma kind::f16) both
// operands are split into three BF16 terms (x = x1 + x2 + x3) and the six products
// x1y1 + x1y2 + x2y1 + x1y3 + x2y2 + x3y1 accumulate in FP32 in tensor memory. B's terms
// are built once per N and cached; A's are formed inside the GEMM from the FP64
// histogram rows (one read of the histogram, no BF16 copy of A in memory).
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "hsr_common.cuh"
#include "hsr_internal.h"

namespace hsr {

namespace {

constexpr int kBM = 128;     // UMMA M
constexpr int kBN = 256;     // UMMA N
constexpr int kBK = 64;      // K per stage: 64 bf16 = 128 B rows (SWIZZLE_128B)
constexpr int kStageA = kBM * kBK * 2;  // 16 KB
constexpr int kStageB = kBN * kBK * 2;  // 32 KB per 256-column half
constexpr int kConvWarps = 8;           // warps forming the A terms (and running the epilogue)
constexpr int kUmmaThreads = 32 * (2 + kConvWarps);
// Shared memory of a CTA computing kNH 256-column halves of its 128-row tile: the three
// A terms of two k-tiles (double buffer, 96 KB) and a ring of B stages (one B term over
// the kNH halves per stage) filling the rest of the 227 KB.
template <int kNH> constexpr int umma_bstages() { return kNH == 1 ? 4 : 2; }
template <int kNH> constexpr int umma_smem() {
    return 2 * 3 * kStageA + umma_bstages<kNH>() * kNH * kStageB + 1024 + 256;
}
constexpr unsigned kStatusSynthTimeout = 1u << 3;

// ------------------------------------------------------------------------------------
// Operand preparation
// ------------------------------------------------------------------------------------

// B^T (K-major): row c of the 2N_pad output columns, column r of the reduction.
__global__ void k_build_bt(const double2 *__restrict__ g, int N, int K, int KK, int KKpad, int NCpad,
                           float *__restrict__ bt) {
    const int64_t idx = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (idx >= int64_t(NCpad) * KKpad) return;
    const int c = int(idx / KKpad), r = int(idx % KKpad);
    float v = 0.f;
    const int KM = kFineMoments * K;
    if (c < 2 * N && r < KK) {
        const int m = c < N ? c : c - N;
        const bool second_half = r >= KM;  // rows of the imaginary histogram part
        const int rr = second_half ? r - KM : r;
        const int d = rr / K, k = rr % K;
        int j = (k - kFineOS * m) % K;
        if (j < 0) j += K;
        const double2 z = g[size_t(d) * K + j];
        if (c < N)
            v = second_half ? float(-z.y) : float(z.x);
        else
            v = second_half ? float(z.x) : float(z.y);
    }
    bt[idx] = v;
}

// x = x1 + x2 + x3 in BF16 (row-major, padded copies) of the FP32 value of x
template <typename T>
__global__ void k_split3(const T *__restrict__ x, int rows, int cols, int ld_in, int rows_pad, int cols_pad,
                         __nv_bfloat16 *__restrict__ o1, __nv_bfloat16 *__restrict__ o2,
                         __nv_bfloat16 *__restrict__ o3) {
    const int64_t idx = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (idx >= int64_t(rows_pad) * cols_pad) return;
    const int r = int(idx / cols_pad), c = int(idx % cols_pad);
    const float v = (r < rows && c < cols) ? float(x[size_t(r) * ld_in + c]) : 0.f;
    const __nv_bfloat16 a = __float2bfloat16_rn(v);
    const float r1 = v - __bfloat162float(a);
    const __nv_bfloat16 b = __float2bfloat16_rn(r1);
    const float r2 = r1 - __bfloat162float(b);
    const __nv_bfloat16 c3 = __float2bfloat16_rn(r2);
    o1[idx] = a;
    o2[idx] = b;
    o3[idx] = c3;
}

// ------------------------------------------------------------------------------------
// CUDA-core FP32 GEMM (cross-check and small batches): C[M x NC] = A[M x KK] * B,
// with B given transposed (bt[NC x KK]).
// ------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_sgemm_nt(const double *__restrict__ a, const float *__restrict__ bt, int M,
                                                  int NC, int KK, int lda, int ldb, float *__restrict__ c, int ldc) {
    __shared__ float As[16][65];
    __shared__ float Bs[16][65];
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    const int m0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
    float acc[4][4] = {};
    for (int k0 = 0; k0 < KK; k0 += 16) {
        for (int t = threadIdx.x; t < 64 * 16; t += 256) {
            const int rr = t / 16, kk = t % 16;
            const int m = m0 + rr, n = n0 + rr, k = k0 + kk;
            As[kk][rr] = (m < M && k < KK) ? float(a[size_t(m) * lda + k]) : 0.f;
            Bs[kk][rr] = (n < NC && k < KK) ? bt[size_t(n) * ldb + k] : 0.f;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < 16; ++kk) {
            float av[4], bv[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) av[i] = As[kk][ty * 4 + i];
#pragma unroll
            for (int j = 0; j < 4; ++j) bv[j] = Bs[kk][tx * 4 + j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int m = m0 + ty * 4 + i, n = n0 + tx * 4 + j;
            if (m < M && n < NC) c[size_t(m) * ldc + n] = acc[i][j];
        }
}

// ------------------------------------------------------------------------------------
// Tensor-core GEMM: tcgen05.mma (kind::f16, BF16 x BF16 -> FP32 in TMEM). A CTA computes
// a 128-row tile over kNH 256-column halves (two FP32 accumulators of 256 TMEM columns
// each for kNH = 2) over a range of k-tiles (split-K over grid.z).
//   warps 2..9 (converters): per k-tile, read the tile's FP64 histogram sums (128 rows x
//     64 columns, one coalesced 512-byte row per warp load), split each into three BF16
//     terms and store them in shared memory in the 128-byte-swizzled K-major layout the
//     MMA descriptors expect (a double buffer of the three term tiles);
//   warp 0 lane 0: TMA loads of B's terms (one term over the kNH halves per ring stage);
//   warp 1 lane 0: per k-tile, for B term j = 1, 2, 3, the MMAs of the A terms i with
//     i + j <= 4 (the six products), then commits that free the B stage and, after the
//     third term, the A buffer.
// Each CTA writes its partial tile to its own slice of the partial buffer, which the
// finalize sums over the slices in order (deterministic). The converter warps run the
// epilogue (TMEM lane quarter = warp % 4, two warps per quarter on half the columns each).
// ------------------------------------------------------------------------------------
struct UmmaParams {
    const double *a;  // fine histograms: M rows of lda FP64, reduction columns [0, K)
    int M, lda, K;    // K: reduction length (multiple of 64)
    float *c;         // partial tiles [grid.z][Mpad][ldc]
    int ldc;          // NCpad
    int64_t slice;    // floats per split-K slice of c
    unsigned *status;
    int chunk;        // k-tiles per CTA along grid.z (split-K)
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait: gives up after ~2^22 polls (each try_wait suspends for a while),
// recording the failure in the status word instead of hanging.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, unsigned *status) {
    for (int i = 0; i < (1 << 22); ++i)
        if (mbar_try_wait(bar, parity)) return true;
    atomicOr(status, kStatusSynthTimeout);
    return false;
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int c0, int c1, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
        "[%4];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(bar)
        : "memory");
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups 1024 B apart.
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= uint64_t((saddr & 0x3FFFF) >> 4);  // start address
    d |= uint64_t(1) << 16;                 // leading byte offset (unused for swizzled K-major)
    d |= uint64_t(1024 >> 4) << 32;         // stride byte offset
    d |= uint64_t(1) << 46;                 // descriptor version
    d |= uint64_t(2) << 61;                 // SWIZZLE_128B
    return d;
}

// Instruction descriptor: FP32 accumulate, BF16 A and B, both K-major, M = 128, N = 256.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(kBN >> 3) << 17) | (uint32_t(kBM >> 4) << 24);

__device__ __forceinline__ void umma(uint32_t tmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.u32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
        "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void umma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// the three BF16 terms of two FP32 values, packed in pairs (first value in the low half)
__device__ __forceinline__ void split3_pair(double x0, double x1, uint32_t &t1, uint32_t &t2, uint32_t &t3) {
    const float v0 = float(x0), v1 = float(x1);
    const __nv_bfloat162 a = __floats2bfloat162_rn(v0, v1);
    const float r0 = v0 - __low2float(a), r1 = v1 - __high2float(a);
    const __nv_bfloat162 b = __floats2bfloat162_rn(r0, r1);
    const __nv_bfloat162 c = __floats2bfloat162_rn(r0 - __low2float(b), r1 - __high2float(b));
    t1 = *reinterpret_cast<const uint32_t *>(&a);
    t2 = *reinterpret_cast<const uint32_t *>(&b);
    t3 = *reinterpret_cast<const uint32_t *>(&c);
}

template <int kNH>
__global__ void __launch_bounds__(kUmmaThreads, 1)
    k_umma_gemm(const __grid_constant__ CUtensorMap tb1, const __grid_constant__ CUtensorMap tb2,
                const __grid_constant__ CUtensorMap tb3, UmmaParams gp) {
    constexpr int kSB = umma_bstages<kNH>();
    constexpr int kBStage = kNH * kStageB;
    constexpr uint32_t kCols = uint32_t(kNH * kBN);  // TMEM columns: 256 or 512
    constexpr int kRowsPerWarp = kBM / kConvWarps;   // 16
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint8_t *abuf = smem;                 // [2][3][kStageA]
    uint8_t *bbuf = smem + 6 * kStageA;   // [kSB][kBStage]
    uint64_t *bars = reinterpret_cast<uint64_t *>(bbuf + kSB * kBStage);
    uint64_t *bfull = bars, *bempty = bars + kSB, *afull = bars + 2 * kSB, *aempty = afull + 2, *done = aempty + 2;
    uint32_t *tmem_holder = reinterpret_cast<uint32_t *>(done + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.x * kBM, n0 = blockIdx.y * int(kCols);
    const int kt0 = blockIdx.z * gp.chunk;
    const int nk = min(gp.K / kBK, kt0 + gp.chunk) - kt0;  // >= 1 by the host's choice of chunk

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_holder)),
                     "r"(kCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int s = 0; s < kSB; ++s) {
            mbar_init(smem_u32(&bfull[s]), 1);
            mbar_init(smem_u32(&bempty[s]), 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(smem_u32(&afull[b]), 32 * kConvWarps);
            mbar_init(smem_u32(&aempty[b]), 1);
        }
        mbar_init(smem_u32(done), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_holder;
    bool ok = true;

    if (warp == 0) {
        if (lane == 0) {
            const CUtensorMap *bm[3] = {&tb1, &tb2, &tb3};
            int n = 0;  // B stages issued
            for (int t = 0; t < nk && ok; ++t) {
                for (int j = 0; j < 3; ++j, ++n) {
                    const int s = n % kSB;
                    if (n >= kSB) ok = mbar_wait(smem_u32(&bempty[s]), uint32_t((n / kSB - 1) & 1), gp.status);
                    if (!ok) break;
                    const uint32_t full = smem_u32(&bfull[s]);
                    mbar_expect_tx(full, kBStage);
#pragma unroll
                    for (int h = 0; h < kNH; ++h)
                        tma_load_2d(smem_u32(bbuf + s * kBStage + h * kStageB), bm[j], (kt0 + t) * kBK,
                                    n0 + h * kBN, full);
                }
            }
            // every load this thread issued has landed before the CTA can exit (bounded)
            for (int s = 0; s < kSB && s < n; ++s) {
                const int last = n - 1 - ((n - 1 - s) % kSB);
                mbar_wait(smem_u32(&bfull[s]), uint32_t((last / kSB) & 1), gp.status);
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            int n = 0;  // B stages consumed
            for (int t = 0; t < nk && ok; ++t) {
                const int ab = t & 1;
                ok = mbar_wait(smem_u32(&afull[ab]), uint32_t((t >> 1) & 1), gp.status);
                if (!ok) break;
                for (int j = 0; j < 3; ++j, ++n) {
                    const int s = n % kSB;
                    ok = mbar_wait(smem_u32(&bfull[s]), uint32_t((n / kSB) & 1), gp.status);
                    if (!ok) break;
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint32_t b0 = smem_u32(bbuf + s * kBStage);
                    for (int i = 0; i + j < 3; ++i) {
                        const uint32_t a0 = smem_u32(abuf + (ab * 3 + i) * kStageA);
#pragma unroll
                        for (int h = 0; h < kNH; ++h) {
#pragma unroll
                            for (int k = 0; k < kBK / 16; ++k)
                                umma(tmem + uint32_t(h * kBN), umma_desc(a0 + 32 * k),
                                     umma_desc(b0 + h * kStageB + 32 * k), (t | j | i | k) ? 1u : 0u);
                        }
                    }
                    umma_commit(smem_u32(&bempty[s]));
                }
                if (ok) umma_commit(smem_u32(&aempty[ab]));
            }
            umma_commit(smem_u32(done));
        }
    } else {
        // converters: lane l holds columns 2l, 2l+1 of a row, i.e. 4 bytes of the row's
        // 16-byte chunk l / 4; the chunk sits at position (l / 4) ^ (row % 8) of the
        // 128-byte row (SWIZZLE_128B: 8-row groups 1024 B apart, tile base 1024-aligned).
        // The loads of k-tile t + 1 are issued before k-tile t is converted, so that a
        // whole tile of the histogram is in flight while the last one is split.
        const int rbase = (warp - 2) * kRowsPerWarp;
        const uint32_t lane_off = uint32_t(lane & 3) * 4;
        double2 cur[kRowsPerWarp], nxt[kRowsPerWarp];
        auto load_tile = [&](int t, double2 (&v)[kRowsPerWarp]) {
            const int col = (kt0 + t) * kBK + 2 * lane;
#pragma unroll
            for (int u = 0; u < kRowsPerWarp; ++u) {
                const int row = m0 + rbase + u;
                v[u] = (row < gp.M) ? __ldg(reinterpret_cast<const double2 *>(gp.a + size_t(row) * gp.lda + col))
                                    : make_double2(0.0, 0.0);
            }
        };
        load_tile(0, cur);
        for (int t = 0; t < nk && ok; ++t) {
            const int ab = t & 1;
            if (t + 1 < nk) load_tile(t + 1, nxt);
            // the buffer is free once the MMAs of k-tile t - 2 completed
            if (t >= 2) ok = mbar_wait(smem_u32(&aempty[ab]), uint32_t(((t >> 1) - 1) & 1), gp.status);
            if (!ok) break;
            uint8_t *at = abuf + ab * 3 * kStageA;
#pragma unroll
            for (int u = 0; u < kRowsPerWarp; ++u) {
                const int r = rbase + u;
                uint32_t w1, w2, w3;
                split3_pair(cur[u].x, cur[u].y, w1, w2, w3);
                const uint32_t off = uint32_t(r) * 128u + ((uint32_t((lane >> 2) ^ (r & 7))) << 4) + lane_off;
                *reinterpret_cast<uint32_t *>(at + off) = w1;
                *reinterpret_cast<uint32_t *>(at + kStageA + off) = w2;
                *reinterpret_cast<uint32_t *>(at + 2 * kStageA + off) = w3;
            }
            // the generic-proxy stores become visible to the tensor cores' async proxy
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            mbar_arrive(smem_u32(&afull[ab]));
#pragma unroll
            for (int u = 0; u < kRowsPerWarp; ++u) cur[u] = nxt[u];
        }
        // epilogue: this warp's 32 TMEM lanes (rows, quarter warp % 4) over its half of the
        // columns (two converter warps share a quarter), 16 columns at a time, into this
        // CTA's slice of the partial buffer
        const int quarter = warp & 3;
        const int cbeg = ((warp - 2) / 4) * int(kCols / 2);
        const bool fin = mbar_wait(smem_u32(done), 0u, gp.status);
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        __syncwarp();
        const int row = m0 + quarter * 32 + lane;
        float *slice = gp.c + size_t(blockIdx.z) * size_t(gp.slice);
        for (int c0 = cbeg; c0 < cbeg + int(kCols / 2); c0 += 16) {
            uint32_t r[16];
            const uint32_t taddr = tmem + (uint32_t(quarter * 32) << 16) + uint32_t(c0);
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                "[%16];"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                  "=r"(r[15])
                : "r"(taddr));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (fin && row < gp.M) {
                float4 *dst = reinterpret_cast<float4 *>(slice + size_t(row) * gp.ldc + n0 + c0);
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    dst[j] = make_float4(__uint_as_float(r[4 * j]), __uint_as_float(r[4 * j + 1]),
                                         __uint_as_float(r[4 * j + 2]), __uint_as_float(r[4 * j + 3]));
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kCols) : "memory");
    }
}

// frame row m: C[p][m] + j C[p][N + m] (the sum of the split-K slices, in slice order),
// divided by the pose's total weight
__global__ void k_synth_finalize(const float *__restrict__ c, int slices, int64_t slice, int P, int N, int ldc,
                                 const int64_t *__restrict__ budget, float sample_weight,
                                 const double *__restrict__ tw, int normalise, float *__restrict__ out) {
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= int64_t(P) * N) return;
    const int p = int(i / N), m = int(i % N);
    float re = 0.f, im = 0.f;
    for (int z = 0; z < slices; ++z) {
        re += c[size_t(z) * slice + size_t(p) * ldc + m];
        im += c[size_t(z) * slice + size_t(p) * ldc + N + m];
    }
    if (normalise) {
        const double w = tw ? tw[p] : double(budget[p]) * double(sample_weight);
        const float inv = 1.f / float(w);
        re *= inv;
        im *= inv;
    }
    out[2 * i] = re;
    out[2 * i + 1] = im;
}

// cuTensorMapEncodeTiled through the driver entry point (no libcuda link-time dependency)
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    }
    return fn;
}

bool make_map(CUtensorMap *map, const void *base, int rows, int cols, int box_rows) {
    EncodeTiledFn fn = encode_fn();
    if (!fn) return false;
    cuuint64_t dims[2] = {cuuint64_t(cols), cuuint64_t(rows)};
    cuuint64_t strides[1] = {cuuint64_t(cols) * 2};
    cuuint32_t box[2] = {cuuint32_t(kBK), cuuint32_t(box_rows)};
    cuuint32_t estr[2] = {1, 1};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

// Twiddle operand B for N range bins, built once and cached by the caller.
int synth_build_operand(SynthOperand &op, int N, cudaStream_t st, std::string &err) {
    const int K = kFineOS * N;
    const int KK = 2 * kFineMoments * K;
    op.N = N;
    op.K = K;
    op.KK = KK;
    op.KKpad = (KK + kBK - 1) / kBK * kBK;
    op.NCpad = (2 * N + kBN - 1) / kBN * kBN;
    // g_d(j), d < 4, j < K, in double on the host: (1/N) sum_n (j w_n)^d e^{j 2 pi (j/8) n / N}
    std::vector<double> g(size_t(kFineMoments) * K * 2);
    const double pi = 3.14159265358979323846;
    for (int j = 0; j < K; ++j) {
        const double x = double(j) / kFineOS;
        double s[kFineMoments][2] = {};
        for (int n = 0; n < N; ++n) {
            const double ang = 2 * pi * x * n / N;
            double zr = std::cos(ang), zi = std::sin(ang);
            const double w = 2 * pi * n / N;
            for (int d = 0; d < kFineMoments; ++d) {
                s[d][0] += zr;
                s[d][1] += zi;
                const double nr = -w * zi, ni = w * zr;  // multiply by j w
                zr = nr;
                zi = ni;
            }
        }
        for (int d = 0; d < kFineMoments; ++d) {
            g[2 * (size_t(d) * K + j)] = s[d][0] / N;
            g[2 * (size_t(d) * K + j) + 1] = s[d][1] / N;
        }
    }
    double2 *dg = nullptr;
    if (!dev_alloc(&dg, g.size() * sizeof(double), err)) return 3;
    cudaMemcpyAsync(dg, g.data(), g.size() * sizeof(double), cudaMemcpyHostToDevice, st);
    const size_t nb = size_t(op.NCpad) * op.KKpad;
    if (!dev_alloc(&op.bt, nb * sizeof(float), err) || !dev_alloc(&op.b1, nb * 2, err) ||
        !dev_alloc(&op.b2, nb * 2, err) || !dev_alloc(&op.b3, nb * 2, err)) {
        cudaFree(dg);
        return 3;
    }
    k_build_bt<<<unsigned((nb + 255) / 256), 256, 0, st>>>(dg, N, K, KK, op.KKpad, op.NCpad, op.bt);
    k_split3<<<unsigned((nb + 255) / 256), 256, 0, st>>>(op.bt, op.NCpad, op.KKpad, op.KKpad, op.NCpad, op.KKpad,
                                                        static_cast<__nv_bfloat16 *>(op.b1),
                                                        static_cast<__nv_bfloat16 *>(op.b2),
                                                        static_cast<__nv_bfloat16 *>(op.b3));
    note_launches(2);
    cudaError_t e = cudaStreamSynchronize(st);
    cudaFree(dg);
    if (e != cudaSuccess) {
        err = std::string("twiddle build: ") + cudaGetErrorString(e);
        return 2;
    }
    return 0;
}

void synth_free_operand(SynthOperand &op) {
    cudaFree(op.bt);
    cudaFree(op.b1);
    cudaFree(op.b2);
    cudaFree(op.b3);
    op = SynthOperand{};
}

namespace {

// The tensor-core launch of one synthesis: 256-column halves per CTA (2 where the padded
// output has them, within the 512 TMEM columns), CTAs along M and N, and split-K over the
// k-tiles so that the grid is about one CTA per SM (each CTA keeping at least 2 k-tiles).
struct UmmaPlan {
    int nh, mtiles, ngroups, split, chunk;
};

UmmaPlan umma_plan(const SynthOperand &op, int P) {
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    UmmaPlan u;
    u.nh = op.NCpad >= 2 * kBN ? 2 : 1;
    u.mtiles = (P + kBM - 1) / kBM;
    u.ngroups = op.NCpad / (u.nh * kBN);
    const int ktiles = op.KKpad / kBK;
    const int tiles = u.mtiles * u.ngroups;
    u.split = std::max(1, std::min(sms / std::max(tiles, 1), ktiles / 2));
    u.chunk = (ktiles + u.split - 1) / u.split;
    u.split = (ktiles + u.chunk - 1) / u.chunk;  // every CTA gets at least one k-tile
    return u;
}

}  // namespace

size_t synth_scratch_bytes(const SynthOperand &op, int P) {
    const int Mpad = (P + kBM - 1) / kBM * kBM;
    const UmmaPlan u = umma_plan(op, P);
    return size_t(std::max(u.split, 1)) * Mpad * op.NCpad * 4 + 256;
}

// fine histograms (P x KK FP64 sums, row stride KK) -> frame rows (P x N complex64)
int synth_run(const SynthOperand &op, const double *fine, int P, void *scratch, int engine, const int64_t *budget,
              float sample_weight, const double *tw, int normalise, float *out_rows, unsigned *status, cudaStream_t st,
              std::string &err) {
    const int Mpad = (P + kBM - 1) / kBM * kBM;
    float *c = static_cast<float *>(scratch);  // the partial slices, [split][Mpad][NCpad]
    const int64_t slice = int64_t(Mpad) * op.NCpad;
    int slices = 1;
    if (engine == 0) {
        if (op.KK != op.KKpad || (reinterpret_cast<uintptr_t>(fine) & 15) != 0) {
            err = "synthesis: histogram rows must be whole k-tiles on a 16-byte boundary";
            return 1;
        }
        CUtensorMap tb[3];
        const void *bs[3] = {op.b1, op.b2, op.b3};
        for (int i = 0; i < 3; ++i) {
            if (!make_map(&tb[i], bs[i], op.NCpad, op.KKpad, kBN)) {
                err = "cuTensorMapEncodeTiled failed";
                return 2;
            }
        }
        const UmmaPlan u = umma_plan(op, P);
        slices = u.split;
        UmmaParams gp{fine, P, op.KK, op.KKpad, c, op.NCpad, slice, status, u.chunk};
        dim3 grid(u.mtiles, u.ngroups, u.split);
        if (u.nh == 2) {
            cudaFuncSetAttribute(k_umma_gemm<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, umma_smem<2>());
            k_umma_gemm<2><<<grid, kUmmaThreads, umma_smem<2>(), st>>>(tb[0], tb[1], tb[2], gp);
        } else {
            cudaFuncSetAttribute(k_umma_gemm<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, umma_smem<1>());
            k_umma_gemm<1><<<grid, kUmmaThreads, umma_smem<1>(), st>>>(tb[0], tb[1], tb[2], gp);
        }
        note_launches(1);
    } else {
        dim3 grid((2 * op.N + 63) / 64, (P + 63) / 64);
        k_sgemm_nt<<<grid, 256, 0, st>>>(fine, op.bt, P, 2 * op.N, op.KK, op.KK, op.KKpad, c, op.NCpad);
        note_launches(1);
    }
    const int64_t n = int64_t(P) * op.N;
    k_synth_finalize<<<unsigned((n + 255) / 256), 256, 0, st>>>(c, slices, slice, P, op.N, op.NCpad, budget,
                                                                sample_weight, tw, normalise, out_rows);
    note_launches(1);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        err = std::string("synthesis launch: ") + cudaGetErrorString(e);
        return 2;
    }
    return 0;
}

}  // namespace hsr
