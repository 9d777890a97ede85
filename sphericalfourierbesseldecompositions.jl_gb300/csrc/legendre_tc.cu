// Legendre contractions on the 5th-generation tensor cores (tcgen05), used
// by the mixed-precision transform.
//
// Split-BF16 products: every FP32 / FP64 operand value x is written as
// x = x0 + x1 + x2 with x0 = bf16(x), x1 = bf16(x - x0), x2 = bf16(x - x0 - x1)
// (24 significant bits), and a product a*b is accumulated as the six terms
// a0b0 + a0b1 + a1b0 + a0b2 + a1b1 + a2b0 (the dropped terms are below
// 2^-24 relative) by tcgen05.mma kind::f16 with FP32 accumulation in TMEM.
//
// Analysis, per block z = (m, parity) and a tile of 128 columns c
// (re/im of the maps):
//   A[l(li)(l+1)/2 + m][c] (+)= sum_r F[parity][m][r][c] * lambda[z][li][r]
// MMA shape M = 128 (columns c), N = rows li padded to 16, K = rings in
// chunks of KC.  The F tile is loaded from global FP32, split by the CTA's
// threads into three K-major BF16 planes in shared memory; the lambda planes
// come pre-split and pre-laid-out from the plan's table with one bulk copy
// (cp.async.bulk, TMA engine) per chunk.  The accumulator lives in TMEM and
// is read back with tcgen05.ld for the epilogue.
//
// Shared-memory operand layout (no swizzle, K-major): 8x8 "core matrices" of
// 128 contiguous bytes (8 rows of 8 bf16); core (g, kk) of a plane with R
// rows sits at ((g * KC/8) + kk) * 128 bytes, so the descriptor's leading
// byte offset (next core along K) is 128 and the stride byte offset (next
// 8-row group) is KC/8 * 128.
//
// Every wait on an mbarrier is bounded; on timeout the CTA records
// ERR_TC_TIMEOUT in the plan's error word, releases its TMEM and returns.
#include <cuda_bf16.h>

#include "sfb_internal.h"
#include "tc_common.cuh"

namespace sfb {
namespace tc {

constexpr int KC = 32;          // rings (K elements) per chunk
constexpr int MTILE = 128;      // columns per CTA (MMA M)
constexpr int NTHREADS = 128;
__device__ __forceinline__ void split3(float x, __nv_bfloat16 &h, __nv_bfloat16 &m, __nv_bfloat16 &l) {
    h = __float2bfloat16_rn(x);
    const float r1 = x - __bfloat162float(h);
    m = __float2bfloat16_rn(r1);
    const float r2 = r1 - __bfloat162float(m);
    l = __float2bfloat16_rn(r2);
}

// FP64 source: the first remainder is formed in FP64 and then carried in FP32
// (exact: x - bf16(x) has at most 16 significant bits above the FP32 floor).
__device__ __forceinline__ void split3(double x, __nv_bfloat16 &h, __nv_bfloat16 &m, __nv_bfloat16 &l) {
    const float xf = (float)x;
    h = __float2bfloat16_rn(xf);
    const float r1 = (float)(x - (double)__bfloat162float(h));
    m = __float2bfloat16_rn(r1);
    const float r2 = r1 - __bfloat162float(m);
    l = __float2bfloat16_rn(r2);
}

// byte offset of element (row, k) in a K-major no-swizzle plane with KC columns
__device__ __forceinline__ uint32_t core_off(int row, int k) {
    return (uint32_t)((((row >> 3) * (KC / 8) + (k >> 3)) << 7) + ((row & 7) << 4) + ((k & 7) << 1));
}

__device__ __forceinline__ int rows_of(int m, int par, int lmax) {
    return (m + par <= lmax) ? (lmax - m - par) / 2 + 1 : 0;
}

__device__ __forceinline__ int pad16(int n) { return (n + 15) & ~15; }

// six split products: (A plane, B plane); product 0 (hi x hi) goes to its own
// accumulator, products 1..5 (the corrections) to a second one.
__constant__ int kPairA[6] = {0, 0, 1, 0, 1, 2};
__constant__ int kPairB[6] = {0, 1, 0, 2, 1, 0};

constexpr int NT8 = 256;   // threads of the chunked kernels (8 warps)

// Double-float accumulation of one chunk's TMEM partials into (hi, lo)
// registers: warp w reads TMEM lanes 32*(w%4).. and the 64 accumulator
// columns [64*(w/4), +64) of the buffer at column `cbase` (hi x hi products)
// and `cbase + 128` (correction products).
__device__ __forceinline__ void chunk_readout(uint32_t tmem, uint32_t cbase, int ncols, float (&hi)[64],
                                              float (&lo)[64]) {
    const int warp = threadIdx.x >> 5;
    const int lq = warp & 3, cg = warp >> 2;
    const uint32_t lane_base = (uint32_t)(lq * 32) << 16;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int col = 64 * cg + 16 * i;
        if (col < ncols) {            // warp-uniform
            float big[16], small[16];
            tmem_ld16(tmem + lane_base + cbase + (uint32_t)col, big);
            tmem_ld16(tmem + lane_base + cbase + 128u + (uint32_t)col, small);
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const float h = hi[16 * i + j], p = big[j];
                const float t = h + p;
                const float bb = t - h;
                lo[16 * i + j] += ((h - (t - bb)) + (p - bb)) + small[j];
                hi[16 * i + j] = t;
            }
        }
    }
}

// 12 MMAs of one 32-wide K chunk: 2 K-steps x 6 split products.
__device__ __forceinline__ void chunk_mma(uint32_t tmem, uint32_t cbase, uint32_t a0, uint32_t planeA, uint32_t b0,
                                          uint32_t planeB, uint32_t idesc) {
    const uint32_t sbo = (KC / 8) * 128;
#pragma unroll
    for (int s = 0; s < KC / 16; ++s) {
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            const uint64_t ad = smem_desc(a0 + kPairA[q] * planeA + s * 256, 128, sbo);
            const uint64_t bd = smem_desc(b0 + kPairB[q] * planeB + s * 256, 128, sbo);
            const uint32_t d = tmem + cbase + (q == 0 ? 0u : 128u);
            const uint32_t acc = (q == 0) ? (s > 0 ? 1u : 0u) : ((s > 0 || q > 1) ? 1u : 0u);
            mma_bf16(d, ad, bd, idesc, acc);
        }
    }
}

// Split two consecutive K values of one operand row into the three planes.
template <typename V>
__device__ __forceinline__ void put_pair(unsigned char *planes, uint32_t planeA, int row, int k, V v0, V v1) {
    __nv_bfloat16 h0, m0, l0, h1, m1, l1;
    split3(v0, h0, m0, l0);
    split3(v1, h1, m1, l1);
    const uint32_t off = core_off(row, k);
    *reinterpret_cast<__nv_bfloat162 *>(planes + off) = __halves2bfloat162(h0, h1);
    *reinterpret_cast<__nv_bfloat162 *>(planes + planeA + off) = __halves2bfloat162(m0, m1);
    *reinterpret_cast<__nv_bfloat162 *>(planes + 2 * planeA + off) = __halves2bfloat162(l0, l1);
}

// Shared memory of the chunked kernels: two stages of (A planes, B planes),
// barriers [0..1] B loaded per stage, [2..3] MMA done per stage, TMEM slot.
struct ChunkSmem {
    unsigned char *A[2], *B[2];
    uint64_t *bars;
    uint32_t *slot;
};

__device__ __forceinline__ ChunkSmem chunk_smem(unsigned char *base, uint32_t planeA, uint32_t planeBmax) {
    ChunkSmem c;
    c.A[0] = base;
    c.A[1] = base + 3 * planeA;
    c.B[0] = base + 6 * planeA;
    c.B[1] = base + 6 * planeA + 3 * planeBmax;
    c.bars = reinterpret_cast<uint64_t *>(base + 6 * planeA + 6 * planeBmax);
    c.slot = reinterpret_cast<uint32_t *>(c.bars + 4);
    return c;
}

__device__ __forceinline__ uint32_t chunk_setup(ChunkSmem &c) {
    const int warp = threadIdx.x >> 5;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(c.slot)),
                     "r"(512)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (threadIdx.x == 0) {
        for (int i = 0; i < 4; ++i) mbar_init(&c.bars[i], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    return *c.slot;
}

__device__ __forceinline__ void chunk_teardown(uint32_t tmem) {
    fence_before();
    __syncthreads();
    if ((threadIdx.x >> 5) == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512) : "memory");
}

// Analysis: grid (column tiles, row halves of 128, blocks z).
__global__ void __launch_bounds__(NT8, 1) k_leg_analysis_tc(const __nv_bfloat16 *__restrict__ lamtc,
                                                            const int64_t *__restrict__ lamtc_off, int lmax, int nrn,
                                                            int nchunks, const float *__restrict__ F, int64_t ncol,
                                                            double *__restrict__ A, int accumulate, int *err) {
    extern __shared__ __align__(1024) unsigned char smem[];
    const int z = blockIdx.z;
    const int m = z >> 1, par = z & 1;
    const int nrows = rows_of(m, par, lmax);
    const int NP = pad16(nrows);
    const int row0 = blockIdx.y * 128;
    if (row0 >= NP) return;
    const int NPc = min(128, NP - row0);
    const int64_t col0 = (int64_t)blockIdx.x * MTILE;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t planeA = MTILE * KC * 2;
    const uint32_t planeB = (uint32_t)NPc * KC * 2;
    ChunkSmem cs = chunk_smem(smem, planeA, 128 * KC * 2);
    const uint32_t tmem = chunk_setup(cs);

    const float *Fz = F + ((int64_t)(par * (lmax + 1) + m) * nrn) * ncol;
    const __nv_bfloat16 *Lz = lamtc + lamtc_off[z];
    const int64_t chunk_elems = 3LL * NP * KC;
    const uint32_t idesc = idesc_bf16(MTILE, NPc);
    // A loads: thread -> column c = tid % 128, ring half kh = tid / 128 (16 rings)
    const int c = tid & 127, kh = tid >> 7;
    const bool cok = col0 + c < ncol;
    float pre[16];
    auto loadA = [&](int kc) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            const int r = kc * KC + kh * 16 + j;
            pre[j] = (cok && r < nrn) ? Fz[(int64_t)r * ncol + col0 + c] : 0.f;
        }
    };
    auto issueB = [&](int kc, int stage) {
        mbar_expect_tx(&cs.bars[stage], 3 * planeB);
        for (int pl = 0; pl < 3; ++pl)
            bulk_g2s(cs.B[stage] + pl * planeB, Lz + kc * chunk_elems + (int64_t)pl * NP * KC + (int64_t)row0 * KC,
                     planeB, &cs.bars[stage]);
    };
    float hi[64], lo[64];
#pragma unroll
    for (int i = 0; i < 64; ++i) hi[i] = lo[i] = 0.f;
    bool ok = true;
    if (tid == 0) issueB(0, 0);
    loadA(0);
    for (int kc = 0; kc < nchunks; ++kc) {
        const int st = kc & 1;
        const uint32_t ph = (uint32_t)((kc >> 1) & 1);      // phase parity of this stage's barriers
#pragma unroll
        for (int j = 0; j < 16; j += 2) put_pair(cs.A[st], planeA, c, kh * 16 + j, pre[j], pre[j + 1]);
        fence_proxy_async();
        __syncthreads();
        if (tid == 0) {
            if (!mbar_wait(&cs.bars[st], ph)) {
                atomicOr(err, ERR_TC_TIMEOUT);
                ok = false;
            } else {
                fence_after();
                chunk_mma(tmem, (uint32_t)st * 256u, smem_u32(cs.A[st]), planeA, smem_u32(cs.B[st]), planeB, idesc);
                mma_commit(&cs.bars[2 + st]);
            }
        }
        if (kc + 1 < nchunks) loadA(kc + 1);
        ok = __syncthreads_and(ok);
        if (!ok) break;
        if (kc > 0) {
            const int sp = st ^ 1;
            if (!mbar_wait(&cs.bars[2 + sp], (uint32_t)(((kc - 1) >> 1) & 1))) {
                atomicOr(err, ERR_TC_TIMEOUT);
                ok = false;
            } else {
                fence_after();
                chunk_readout(tmem, (uint32_t)sp * 256u, NPc, hi, lo);
            }
        }
        fence_before();
        ok = __syncthreads_and(ok);
        if (!ok) break;
        if (tid == 0 && kc + 1 < nchunks) issueB(kc + 1, st ^ 1);
    }
    if (ok) {
        const int sl = (nchunks - 1) & 1;
        if (!mbar_wait(&cs.bars[2 + sl], (uint32_t)(((nchunks - 1) >> 1) & 1))) {
            atomicOr(err, ERR_TC_TIMEOUT);
            ok = false;
        } else {
            fence_after();
            chunk_readout(tmem, (uint32_t)sl * 256u, NPc, hi, lo);
        }
    }
    if (ok) {
        const int lq = warp & 3, cg = warp >> 2;
        const int64_t cc = col0 + lq * 32 + lane;
        if (cc < ncol) {
#pragma unroll
            for (int i = 0; i < 64; ++i) {
                const int li = row0 + 64 * cg + i;
                if (64 * cg + i < NPc && li < nrows) {
                    const int l = m + par + 2 * li;
                    double *d = A + ((int64_t)l * (l + 1) / 2 + m) * ncol + cc;
                    const double v = (double)hi[i] + (double)lo[i];
                    *d = accumulate ? *d + v : v;
                }
            }
        }
    }
    chunk_teardown(tmem);
}

// Pre-split lambda table for the analysis kernel: block z, chunk kc, plane p,
// row li < NP, ring k < KC in the core-matrix layout above (zero padding).
__global__ void k_build_lamtc(const double *__restrict__ lam, const int64_t *lam_off, int lmax, int nrn, int nchunks,
                              const int64_t *lamtc_off, __nv_bfloat16 *lamtc) {
    const int z = blockIdx.y;
    const int m = z >> 1, par = z & 1;
    const int nrows = rows_of(m, par, lmax);
    if (nrows == 0) return;
    const int NP = pad16(nrows);
    const int64_t total = (int64_t)NP * nchunks * KC;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int li = (int)(idx / ((int64_t)nchunks * KC));
        const int rr = (int)(idx - (int64_t)li * nchunks * KC);
        const int kc = rr / KC, k = rr % KC;
        double v = 0.0;
        if (li < nrows && rr < nrn) v = lam[lam_off[z] + (int64_t)li * nrn + rr];
        const __nv_bfloat16 h = __double2bfloat16(v);
        const double r1 = v - (double)__bfloat162float(h);
        const __nv_bfloat16 mm = __double2bfloat16(r1);
        const double r2 = r1 - (double)__bfloat162float(mm);
        const __nv_bfloat16 lo = __double2bfloat16(r2);
        const int64_t chunk_elems = 3LL * NP * KC;
        const int64_t base = lamtc_off[z] + (int64_t)kc * chunk_elems;
        const int64_t e = core_off(li, k) >> 1;
        lamtc[base + e] = h;
        lamtc[base + (int64_t)NP * KC + e] = mm;
        lamtc[base + 2LL * NP * KC + e] = lo;
    }
}

// Synthesis, per block z = (m, parity), ring tile nt (NT = 128 rings) and a
// tile of 128 columns:
//   G[parity][m][r][c] = sum_li lambda[z][li][r] * A[l(li)(l+1)/2 + m][c]
// MMA shape M = 128 (columns), N = NT rings, K = rows li in chunks of KC, with
// the same chunked double-float accumulation as the analysis.
__global__ void __launch_bounds__(NT8, 1) k_leg_synthesis_tc(const __nv_bfloat16 *__restrict__ lamts,
                                                             const int64_t *__restrict__ lamts_off, int lmax, int nrn,
                                                             int NT, const double *__restrict__ A, int64_t ncol,
                                                             float *__restrict__ G, int *err) {
    extern __shared__ __align__(1024) unsigned char smem[];
    const int z = blockIdx.z;
    const int m = z >> 1, par = z & 1;
    const int nrows = rows_of(m, par, lmax);
    const int nt = blockIdx.y;
    const int r0 = nt * NT;
    const int64_t col0 = (int64_t)blockIdx.x * MTILE;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    float *Gz = G + ((int64_t)(par * (lmax + 1) + m) * nrn) * ncol;
    if (nrows == 0) {      // no l for this (m, parity): the block is zero
        for (int rr = warp; rr < NT; rr += NT8 / 32) {
            const int r = r0 + rr;
            if (r >= nrn) break;
            for (int64_t cc = col0 + lane; cc < col0 + MTILE && cc < ncol; cc += 32) Gz[(int64_t)r * ncol + cc] = 0.f;
        }
        return;
    }
    const int nK = (nrows + KC - 1) / KC;
    const uint32_t planeA = MTILE * KC * 2;
    const uint32_t planeB = (uint32_t)NT * KC * 2;
    ChunkSmem cs = chunk_smem(smem, planeA, planeB);
    const uint32_t tmem = chunk_setup(cs);
    const __nv_bfloat16 *Lz = lamts + lamts_off[z] + (int64_t)nt * nK * 3 * NT * KC;
    const uint32_t idesc = idesc_bf16(MTILE, NT);
    const int c = tid & 127, kh = tid >> 7;
    const bool cok = col0 + c < ncol;
    double pre[16];
    auto loadA = [&](int kc) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            const int li = kc * KC + kh * 16 + j;
            double v = 0.0;
            if (cok && li < nrows) {
                const int l = m + par + 2 * li;
                v = A[((int64_t)l * (l + 1) / 2 + m) * ncol + col0 + c];
            }
            pre[j] = v;
        }
    };
    auto issueB = [&](int kc, int stage) {
        mbar_expect_tx(&cs.bars[stage], 3 * planeB);
        bulk_g2s(cs.B[stage], Lz + (int64_t)kc * 3 * NT * KC, 3 * planeB, &cs.bars[stage]);
    };
    float hi[64], lo[64];
#pragma unroll
    for (int i = 0; i < 64; ++i) hi[i] = lo[i] = 0.f;
    bool ok = true;
    if (tid == 0) issueB(0, 0);
    loadA(0);
    for (int kc = 0; kc < nK; ++kc) {
        const int st = kc & 1;
        const uint32_t ph = (uint32_t)((kc >> 1) & 1);
#pragma unroll
        for (int j = 0; j < 16; j += 2) put_pair(cs.A[st], planeA, c, kh * 16 + j, pre[j], pre[j + 1]);
        fence_proxy_async();
        __syncthreads();
        if (tid == 0) {
            if (!mbar_wait(&cs.bars[st], ph)) {
                atomicOr(err, ERR_TC_TIMEOUT);
                ok = false;
            } else {
                fence_after();
                chunk_mma(tmem, (uint32_t)st * 256u, smem_u32(cs.A[st]), planeA, smem_u32(cs.B[st]), planeB, idesc);
                mma_commit(&cs.bars[2 + st]);
            }
        }
        if (kc + 1 < nK) loadA(kc + 1);
        ok = __syncthreads_and(ok);
        if (!ok) break;
        if (kc > 0) {
            const int sp = st ^ 1;
            if (!mbar_wait(&cs.bars[2 + sp], (uint32_t)(((kc - 1) >> 1) & 1))) {
                atomicOr(err, ERR_TC_TIMEOUT);
                ok = false;
            } else {
                fence_after();
                chunk_readout(tmem, (uint32_t)sp * 256u, NT, hi, lo);
            }
        }
        fence_before();
        ok = __syncthreads_and(ok);
        if (!ok) break;
        if (tid == 0 && kc + 1 < nK) issueB(kc + 1, st ^ 1);
    }
    if (ok) {
        const int sl = (nK - 1) & 1;
        if (!mbar_wait(&cs.bars[2 + sl], (uint32_t)(((nK - 1) >> 1) & 1))) {
            atomicOr(err, ERR_TC_TIMEOUT);
            ok = false;
        } else {
            fence_after();
            chunk_readout(tmem, (uint32_t)sl * 256u, NT, hi, lo);
        }
    }
    if (ok) {
        const int lq = warp & 3, cg = warp >> 2;
        const int64_t cc = col0 + lq * 32 + lane;
        if (cc < ncol) {
#pragma unroll
            for (int i = 0; i < 64; ++i) {
                const int r = r0 + 64 * cg + i;
                if (64 * cg + i < NT && r < nrn) Gz[(int64_t)r * ncol + cc] = hi[i] + lo[i];
            }
        }
    }
    chunk_teardown(tmem);
}

// Synthesis table: block z, ring tile nt, chunk kc, plane p, ring rr < NT,
// row k < KC in the core-matrix layout (N = rings, K = rows li).
__global__ void k_build_lamts(const double *__restrict__ lam, const int64_t *lam_off, int lmax, int nrn, int NT,
                              const int64_t *lamts_off, __nv_bfloat16 *lamts) {
    const int z = blockIdx.y;
    const int m = z >> 1, par = z & 1;
    const int nrows = rows_of(m, par, lmax);
    if (nrows == 0) return;
    const int nK = (nrows + KC - 1) / KC;
    const int ntiles = (nrn + NT - 1) / NT;
    const int64_t total = (int64_t)ntiles * NT * nK * KC;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t rg = idx / ((int64_t)nK * KC);          // global ring slot (tile-major)
        const int kk = (int)(idx - rg * nK * KC);
        const int nt = (int)(rg / NT), rr = (int)(rg % NT);
        const int kc = kk / KC, k = kk % KC;
        const int r = nt * NT + rr, li = kc * KC + k;
        double v = 0.0;
        if (r < nrn && li < nrows) v = lam[lam_off[z] + (int64_t)li * nrn + r];
        const __nv_bfloat16 h = __double2bfloat16(v);
        const double r1 = v - (double)__bfloat162float(h);
        const __nv_bfloat16 mm = __double2bfloat16(r1);
        const double r2 = r1 - (double)__bfloat162float(mm);
        const __nv_bfloat16 lo = __double2bfloat16(r2);
        const int64_t plane = (int64_t)NT * KC;
        const int64_t base = lamts_off[z] + ((int64_t)nt * nK + kc) * 3 * plane;
        const int64_t e = core_off(rr, k) >> 1;
        lamts[base + e] = h;
        lamts[base + plane + e] = mm;
        lamts[base + 2 * plane + e] = lo;
    }
}

// Self-test of the bounded waits: one CTA waits on an mbarrier that nothing
// arrives at; the wait gives up after SPIN_LIMIT polls and records the error.
__global__ void k_selftest_wait(int *err) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0 && !mbar_wait(&bar, 0)) atomicOr(err, ERR_TC_TIMEOUT);
}

}  // namespace tc

int tc_chunks(const Plan &p) { return (int)((p.nrn + tc::KC - 1) / tc::KC); }

int tc_np_max(const Plan &p) {
    const int nr = p.lmax / 2 + 1;
    return (nr + 15) & ~15;
}

static size_t chunk_smem_bytes(int nb_rows) {
    return 6 * (size_t)tc::MTILE * tc::KC * 2 + 6 * (size_t)nb_rows * tc::KC * 2 + 64;
}

// offsets (in bf16 elements) of every block of the analysis table; returns the total
int64_t tc_table_offsets(const Plan &p, std::vector<int64_t> &off) {
    const int nch = tc_chunks(p);
    off.assign(2 * (p.lmax + 1) + 1, 0);
    int64_t o = 0;
    for (int z = 0; z < 2 * (p.lmax + 1); ++z) {
        const int m = z >> 1, par = z & 1;
        const int nrows = (m + par <= p.lmax) ? (p.lmax - m - par) / 2 + 1 : 0;
        off[z] = o;
        if (nrows > 0) o += 3LL * ((nrows + 15) & ~15) * nch * tc::KC;
    }
    off[2 * (p.lmax + 1)] = o;
    return o;
}

void launch_build_lamtc(const Plan &p, cudaStream_t st) {
    dim3 grid(64, (unsigned)(2 * (p.lmax + 1)));
    tc::k_build_lamtc<<<grid, 256, 0, st>>>(p.d_lam, p.d_lam_off, p.lmax, (int)p.nrn, tc_chunks(p), p.d_lamtc_off,
                                            (__nv_bfloat16 *)p.d_lamtc);
    note_launch();
}

void launch_leg_analysis_tc(const Plan &p, const float *F, int64_t ncol, double *A, bool accumulate, cudaStream_t st) {
    const size_t smem = chunk_smem_bytes(128);
    set_smem(tc::k_leg_analysis_tc, smem);
    const int nhalf = (tc_np_max(p) + 127) / 128;
    dim3 grid((unsigned)((ncol + tc::MTILE - 1) / tc::MTILE), (unsigned)nhalf, (unsigned)(2 * (p.lmax + 1)));
    tc::k_leg_analysis_tc<<<grid, tc::NT8, smem, st>>>((const __nv_bfloat16 *)p.d_lamtc, p.d_lamtc_off, p.lmax,
                                                      (int)p.nrn, tc_chunks(p), F, ncol, A, accumulate ? 1 : 0,
                                                      p.d_err);
    note_launch();
}

}  // namespace sfb

namespace sfb {

int tc_synth_nt(const Plan &p) {
    const int nrn = (int)p.nrn;
    const int nt16 = (nrn + 15) & ~15;
    return nt16 < 128 ? nt16 : 128;
}

int64_t tc_synth_table_offsets(const Plan &p, std::vector<int64_t> &off) {
    const int NT = tc_synth_nt(p);
    const int ntiles = (int)((p.nrn + NT - 1) / NT);
    off.assign(2 * (p.lmax + 1) + 1, 0);
    int64_t o = 0;
    for (int z = 0; z < 2 * (p.lmax + 1); ++z) {
        const int m = z >> 1, par = z & 1;
        const int nrows = (m + par <= p.lmax) ? (p.lmax - m - par) / 2 + 1 : 0;
        off[z] = o;
        if (nrows > 0) o += 3LL * NT * ((nrows + tc::KC - 1) / tc::KC) * tc::KC * ntiles;
    }
    off[2 * (p.lmax + 1)] = o;
    return o;
}

void launch_build_lamts(const Plan &p, cudaStream_t st) {
    dim3 grid(64, (unsigned)(2 * (p.lmax + 1)));
    tc::k_build_lamts<<<grid, 256, 0, st>>>(p.d_lam, p.d_lam_off, p.lmax, (int)p.nrn, tc_synth_nt(p), p.d_lamts_off,
                                            (__nv_bfloat16 *)p.d_lamts);
    note_launch();
}

void launch_leg_synthesis_tc(const Plan &p, const double *A, int64_t ncol, float *G, cudaStream_t st) {
    const int NT = tc_synth_nt(p);
    const size_t smem = chunk_smem_bytes(NT);
    set_smem(tc::k_leg_synthesis_tc, smem);
    dim3 grid((unsigned)((ncol + tc::MTILE - 1) / tc::MTILE), (unsigned)((p.nrn + NT - 1) / NT),
              (unsigned)(2 * (p.lmax + 1)));
    tc::k_leg_synthesis_tc<<<grid, tc::NT8, smem, st>>>((const __nv_bfloat16 *)p.d_lamts, p.d_lamts_off, p.lmax,
                                                       (int)p.nrn, NT, A, ncol, G, p.d_err);
    note_launch();
}

}  // namespace sfb

extern "C" int sfb_selftest_wait_timeout(void) {
    int *d = nullptr;
    if (cudaMalloc(&d, sizeof(int)) != cudaSuccess) {
        cudaGetLastError();
        return sfb::fail(SFB_ECUDA, "no CUDA device available");
    }
    cudaMemset(d, 0, sizeof(int));
    sfb::tc::k_selftest_wait<<<1, 32>>>(d);
    sfb::note_launch();
    int h = 0;
    const cudaError_t e = cudaMemcpy(&h, d, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return sfb::fail(SFB_ECUDA, cudaGetErrorString(e));
    if (h & sfb::ERR_TC_TIMEOUT) return sfb::fail(SFB_ETIMEOUT, "self-test: bounded mbarrier wait expired as expected");
    return SFB_OK;
}
