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
// x1y1 + x1y2 + x2y1 + x1y3 + x2y2 + x3y1 accumulate in FP32 in tensor memory.
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
// pipeline depth for a CTA computing kNH 256-column halves of its 128-row tile: the ring
// of (A, kNH x B) stages within the 227 KB of shared memory
template <int kNH> constexpr int umma_stages() { return kNH == 1 ? 4 : 2; }
template <int kNH> constexpr int umma_smem() { return umma_stages<kNH>() * (kStageA + kNH * kStageB) + 1024 + 256; }
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

// The same split for the A operand, eight columns per thread: row r of the padded
// output (blockIdx.y), columns 8 (blockIdx.x * blockDim.x + threadIdx.x) onwards; the
// eight FP64 sums are read as four 16-byte loads and each term is stored as one 16-byte
// chunk. cols_pad is a multiple of 8; every element of a chunk is either inside
// [rows) x [cols) or padding (cols, the histogram length 64 N, is a multiple of 8).
__global__ void k_split3_v8(const double *__restrict__ x, int rows, int cols, int ld_in, int cols_pad,
                            __nv_bfloat16 *__restrict__ o1, __nv_bfloat16 *__restrict__ o2,
                            __nv_bfloat16 *__restrict__ o3) {
    const int r = blockIdx.y;
    const int c = 8 * (blockIdx.x * blockDim.x + threadIdx.x);
    if (c >= cols_pad) return;
    float v[8];
    if (r < rows && c < cols) {
        const double2 *src = reinterpret_cast<const double2 *>(x + size_t(r) * ld_in + c);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const double2 d = __ldg(src + j);
            v[2 * j] = float(d.x);
            v[2 * j + 1] = float(d.y);
        }
    } else {
#pragma unroll
        for (int j = 0; j < 8; ++j) v[j] = 0.f;
    }
    __align__(16) __nv_bfloat16 t1[8], t2[8], t3[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        t1[j] = __float2bfloat16_rn(v[j]);
        const float r1 = v[j] - __bfloat162float(t1[j]);
        t2[j] = __float2bfloat16_rn(r1);
        const float r2 = r1 - __bfloat162float(t2[j]);
        t3[j] = __float2bfloat16_rn(r2);
    }
    const size_t o = size_t(r) * cols_pad + c;
    *reinterpret_cast<uint4 *>(o1 + o) = *reinterpret_cast<const uint4 *>(t1);
    *reinterpret_cast<uint4 *>(o2 + o) = *reinterpret_cast<const uint4 *>(t2);
    *reinterpret_cast<uint4 *>(o3 + o) = *reinterpret_cast<const uint4 *>(t3);
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
// Tensor-core GEMM: tcgen05.mma (kind::f16, BF16 x BF16 -> FP32 in TMEM), operands
// staged by TMA (128-byte swizzle). A CTA computes a 128-row tile over kNH 256-column
// halves (two FP32 accumulators of 256 TMEM columns each for kNH = 2), so its A tile is
// fetched once for both halves. Its k-iterations are (k-tile, split product) pairs in
// k-major order: the products x_i y_j of one k-tile follow each other, and the A term
// tile a product shares with the previous one comes from L2. Split-K over grid.z; each
// CTA writes its partial tile to its own slice of the partial buffer, which the
// finalize sums over the slices in order (deterministic).
// Warp 0 lane 0 issues TMA, warp 1 lane 0 issues MMA, all four warps run the epilogue.
// ------------------------------------------------------------------------------------
struct UmmaParams {
    int M, NC, KK;  // KK: padded reduction length of one product (multiple of 64)
    float *c;       // partial tiles [grid.z][Mpad][ldc]
    int ldc;        // NCpad
    int64_t slice;  // floats per split-K slice of c
    unsigned *status;
    int chunk;      // k-iterations per CTA along grid.z (split-K)
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

template <int kNH>
__global__ void __launch_bounds__(128, 1)
    k_umma_gemm(const __grid_constant__ CUtensorMap ta1, const __grid_constant__ CUtensorMap ta2,
                const __grid_constant__ CUtensorMap ta3, const __grid_constant__ CUtensorMap tb1,
                const __grid_constant__ CUtensorMap tb2, const __grid_constant__ CUtensorMap tb3, UmmaParams gp) {
    constexpr int kS = umma_stages<kNH>();
    constexpr int kStage = kStageA + kNH * kStageB;
    constexpr uint32_t kCols = uint32_t(kNH * kBN);  // TMEM columns: 256 or 512
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + kS * kStage);  // full[kS], empty[kS], done
    uint32_t *tmem_holder = reinterpret_cast<uint32_t *>(bars + 2 * kS + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.x * kBM, n0 = blockIdx.y * int(kCols);

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_holder)),
                     "r"(kCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int st = 0; st < 2 * kS + 1; ++st) mbar_init(smem_u32(&bars[st]), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_holder;

    const int ktiles = gp.KK / kBK;
    const int it0 = blockIdx.z * gp.chunk;
    const int it1 = min(6 * ktiles, it0 + gp.chunk);
    const int total = it1 - it0;  // >= 1 by the host's choice of chunk
    // products x_i y_j of the three-term splits: (1,1) (1,2) (2,1) (1,3) (2,2) (3,1)
    const int pa[6] = {0, 0, 1, 0, 1, 2};
    const int pb[6] = {0, 1, 0, 2, 1, 0};
    bool ok = true;

    if (warp == 0 && lane == 0) {
        const CUtensorMap *am[3] = {&ta1, &ta2, &ta3};
        const CUtensorMap *bm[3] = {&tb1, &tb2, &tb3};
        for (int it = 0; it < total && ok; ++it) {
            const int st = it % kS, round = it / kS;
            if (it >= kS) ok = mbar_wait(smem_u32(&bars[kS + st]), uint32_t((round - 1) & 1), gp.status);
            if (!ok) break;
            const uint32_t full = smem_u32(&bars[st]);
            mbar_expect_tx(full, kStage);
            const int kt = (it0 + it) / 6, pair = (it0 + it) % 6;  // k-major: products of a k-tile adjacent
            uint8_t *stage = smem + st * kStage;
            tma_load_2d(smem_u32(stage), am[pa[pair]], kt * kBK, m0, full);
#pragma unroll
            for (int h = 0; h < kNH; ++h)
                tma_load_2d(smem_u32(stage + kStageA + h * kStageB), bm[pb[pair]], kt * kBK, n0 + h * kBN, full);
        }
    } else if (warp == 1 && lane == 0) {
        for (int it = 0; it < total && ok; ++it) {
            const int st = it % kS, round = it / kS;
            ok = mbar_wait(smem_u32(&bars[st]), uint32_t(round & 1), gp.status);
            if (!ok) break;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t a0 = smem_u32(smem + st * kStage);
#pragma unroll
            for (int h = 0; h < kNH; ++h) {
                const uint32_t b0 = a0 + kStageA + h * kStageB;
#pragma unroll
                for (int k = 0; k < kBK / 16; ++k)
                    umma(tmem + uint32_t(h * kBN), umma_desc(a0 + 32 * k), umma_desc(b0 + 32 * k),
                         (it > 0 || k > 0) ? 1u : 0u);
            }
            umma_commit(smem_u32(&bars[kS + st]));
        }
        umma_commit(smem_u32(&bars[2 * kS]));
    }
    __syncwarp();
    // epilogue: each warp reads its 32 TMEM lanes (rows), 16 columns at a time, into this
    // CTA's slice of the partial buffer
    const bool done = mbar_wait(smem_u32(&bars[2 * kS]), 0u, gp.status);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    __syncwarp();
    const int row = m0 + warp * 32 + lane;
    float *slice = gp.c + size_t(blockIdx.z) * size_t(gp.slice);
    for (int c0 = 0; c0 < int(kCols); c0 += 16) {
        uint32_t r[16];
        const uint32_t taddr = tmem + (uint32_t(warp * 32) << 16) + uint32_t(c0);
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
            : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (done && row < gp.M) {
            float4 *dst = reinterpret_cast<float4 *>(slice + size_t(row) * gp.ldc + n0 + c0);
#pragma unroll
            for (int j = 0; j < 4; ++j)
                dst[j] = make_float4(__uint_as_float(r[4 * j]), __uint_as_float(r[4 * j + 1]),
                                     __uint_as_float(r[4 * j + 2]), __uint_as_float(r[4 * j + 3]));
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
// output has them, within the 512 TMEM columns), CTAs along M and N, and split-K so that
// the grid is about one CTA per SM (each CTA keeping at least 8 k-iterations).
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
    const int iters = 6 * (op.KKpad / kBK);
    const int tiles = u.mtiles * u.ngroups;
    u.split = std::max(1, std::min(sms / std::max(tiles, 1), iters / 8));
    u.chunk = (iters + u.split - 1) / u.split;
    u.split = (iters + u.chunk - 1) / u.chunk;  // every CTA gets at least one k-iteration
    return u;
}

}  // namespace

size_t synth_scratch_bytes(const SynthOperand &op, int P) {
    const int Mpad = (P + kBM - 1) / kBM * kBM;
    const UmmaPlan u = umma_plan(op, P);
    return size_t(Mpad) * op.KKpad * 2 * 3 + size_t(std::max(u.split, 1)) * Mpad * op.NCpad * 4 + 3 * 256;
}

// fine histograms (P x KK FP64 sums, row stride KK) -> frame rows (P x N complex64)
int synth_run(const SynthOperand &op, const double *fine, int P, void *scratch, int engine, const int64_t *budget,
              float sample_weight, const double *tw, int normalise, float *out_rows, unsigned *status, cudaStream_t st,
              std::string &err) {
    const int Mpad = (P + kBM - 1) / kBM * kBM;
    char *p = static_cast<char *>(scratch);
    auto take = [&](size_t bytes) {
        char *r = p;
        p += (bytes + 255) & ~size_t(255);
        return r;
    };
    const size_t na = size_t(Mpad) * op.KKpad;
    __nv_bfloat16 *a1 = reinterpret_cast<__nv_bfloat16 *>(take(na * 2));
    __nv_bfloat16 *a2 = reinterpret_cast<__nv_bfloat16 *>(take(na * 2));
    __nv_bfloat16 *a3 = reinterpret_cast<__nv_bfloat16 *>(take(na * 2));
    float *c = reinterpret_cast<float *>(p);  // the partial slices, [split][Mpad][NCpad]
    const int64_t slice = int64_t(Mpad) * op.NCpad;
    int slices = 1;
    if (engine == 0) {
        const dim3 sg(unsigned((op.KKpad / 8 + 255) / 256), unsigned(Mpad));
        k_split3_v8<<<sg, 256, 0, st>>>(fine, P, op.KK, op.KK, op.KKpad, a1, a2, a3);
        CUtensorMap ta[3], tb[3];
        const void *as[3] = {a1, a2, a3};
        const void *bs[3] = {op.b1, op.b2, op.b3};
        for (int i = 0; i < 3; ++i) {
            if (!make_map(&ta[i], as[i], Mpad, op.KKpad, kBM) || !make_map(&tb[i], bs[i], op.NCpad, op.KKpad, kBN)) {
                err = "cuTensorMapEncodeTiled failed";
                return 2;
            }
        }
        const UmmaPlan u = umma_plan(op, P);
        slices = u.split;
        UmmaParams gp{P, 2 * op.N, op.KKpad, c, op.NCpad, slice, status, u.chunk};
        dim3 grid(u.mtiles, u.ngroups, u.split);
        if (u.nh == 2) {
            cudaFuncSetAttribute(k_umma_gemm<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, umma_smem<2>());
            k_umma_gemm<2><<<grid, 128, umma_smem<2>(), st>>>(ta[0], ta[1], ta[2], tb[0], tb[1], tb[2], gp);
        } else {
            cudaFuncSetAttribute(k_umma_gemm<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, umma_smem<1>());
            k_umma_gemm<1><<<grid, 128, umma_smem<1>(), st>>>(ta[0], ta[1], ta[2], tb[0], tb[1], tb[2], gp);
        }
        note_launches(2);
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
