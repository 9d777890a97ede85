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

namespace sfb {
namespace tc {

constexpr int KC = 32;          // rings (K elements) per chunk
constexpr int MTILE = 128;      // columns per CTA (MMA M)
constexpr int NTHREADS = 128;
constexpr uint32_t SPIN_LIMIT = 1u << 20;   // ~1 s of try_wait polling

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;      // descriptor version for the sm_100 family; no swizzle, base offset 0
    return d;
}

// kind::f16 instruction descriptor: BF16 x BF16 -> F32, both operands K-major.
__device__ __forceinline__ uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// Bounded wait for the given phase parity; false on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
    const uint32_t a = smem_u32(bar);
    for (uint32_t it = 0; it < SPIN_LIMIT; ++it) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accum) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
            tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accum)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void split3(float x, __nv_bfloat16 &h, __nv_bfloat16 &m, __nv_bfloat16 &l) {
    h = __float2bfloat16_rn(x);
    const float r1 = x - __bfloat162float(h);
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

// six split products: (A plane, B plane)
__constant__ int kPairA[6] = {0, 0, 1, 0, 1, 2};
__constant__ int kPairB[6] = {0, 1, 0, 2, 1, 0};

__global__ void __launch_bounds__(NTHREADS) k_leg_analysis_tc(const __nv_bfloat16 *__restrict__ lamtc,
                                                               const int64_t *__restrict__ lamtc_off, int lmax,
                                                               int nrn, int nchunks, const float *__restrict__ F,
                                                               int64_t ncol, float *__restrict__ A, int accumulate,
                                                               int np_max, int *err) {
    extern __shared__ __align__(1024) unsigned char smem[];
    const int z = blockIdx.z;
    const int m = z >> 1, par = z & 1;
    const int nrows = rows_of(m, par, lmax);
    if (nrows == 0) return;
    const int NP = pad16(nrows);
    const int64_t col0 = (int64_t)blockIdx.x * MTILE;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    const uint32_t planeA = MTILE * KC * 2;                  // bytes per A plane
    const uint32_t planeB = (uint32_t)np_max * KC * 2;       // bytes per B plane (allocation)
    unsigned char *sA = smem;                                // 3 planes
    unsigned char *sB = smem + 3 * planeA;                   // 3 planes of NP rows (packed by the table)
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + 3 * planeA + 3 * planeB);   // [0] B loaded, [1] MMA done
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 2);

    const uint32_t ncols_tmem = NP <= 32 ? 32 : (NP <= 64 ? 64 : (NP <= 128 ? 128 : 256));
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(ncols_tmem)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tmem_slot;

    const float *Fz = F + ((int64_t)(par * (lmax + 1) + m) * nrn) * ncol;
    const __nv_bfloat16 *Lz = lamtc + lamtc_off[z];
    const uint32_t chunkB = 3u * (uint32_t)NP * KC * 2;      // bytes of one pre-split chunk of this block
    const uint32_t idesc = idesc_bf16(MTILE, NP);
    const uint32_t sbo = (KC / 8) * 128;
    bool ok = true;

    for (int kc = 0; kc < nchunks && ok; ++kc) {
        const uint32_t phase = (uint32_t)(kc & 1);
        if (tid == 0) {
            mbar_expect_tx(&bars[0], chunkB);
            bulk_g2s(sB, Lz + (int64_t)kc * (chunkB / 2), chunkB, &bars[0]);
        }
        // A planes: thread tid owns column c = tid; two rings per 32-bit store
        const int c = tid;
        const bool cok = col0 + c < ncol;
#pragma unroll 4
        for (int k = 0; k < KC; k += 2) {
            const int r0 = kc * KC + k;
            float v0 = 0.f, v1 = 0.f;
            if (cok) {
                if (r0 < nrn) v0 = Fz[(int64_t)r0 * ncol + col0 + c];
                if (r0 + 1 < nrn) v1 = Fz[(int64_t)(r0 + 1) * ncol + col0 + c];
            }
            __nv_bfloat16 h0, m0, l0, h1, m1, l1;
            split3(v0, h0, m0, l0);
            split3(v1, h1, m1, l1);
            const uint32_t off = core_off(c, k);
            *reinterpret_cast<__nv_bfloat162 *>(sA + off) = __halves2bfloat162(h0, h1);
            *reinterpret_cast<__nv_bfloat162 *>(sA + planeA + off) = __halves2bfloat162(m0, m1);
            *reinterpret_cast<__nv_bfloat162 *>(sA + 2 * planeA + off) = __halves2bfloat162(l0, l1);
        }
        fence_proxy_async();
        __syncthreads();
        if (tid == 0) {
            if (!mbar_wait(&bars[0], phase)) {
                atomicOr(err, ERR_TC_TIMEOUT);
                ok = false;
            } else {
                fence_after();
                const uint32_t a0 = smem_u32(sA), b0 = smem_u32(sB);
                const uint32_t planeBz = (uint32_t)NP * KC * 2;
#pragma unroll
                for (int s = 0; s < KC / 16; ++s) {
#pragma unroll
                    for (int q = 0; q < 6; ++q) {
                        const uint64_t ad = smem_desc(a0 + kPairA[q] * planeA + s * 256, 128, sbo);
                        const uint64_t bd = smem_desc(b0 + kPairB[q] * planeBz + s * 256, 128, sbo);
                        mma_bf16(tmem, ad, bd, idesc, (kc > 0 || s > 0 || q > 0) ? 1u : 0u);
                    }
                }
                mma_commit(&bars[1]);
            }
        }
        // every thread waits for the chunk's MMAs before its smem is reused
        ok = __syncthreads_and(ok);
        if (!ok) break;
        if (!mbar_wait(&bars[1], phase)) {
            atomicOr(err, ERR_TC_TIMEOUT);
            ok = false;
        }
        ok = __syncthreads_and(ok);
    }
    fence_after();
    if (ok) {
        const int64_t c = col0 + warp * 32 + lane;
        for (int n0 = 0; n0 < NP; n0 += 16) {
            float v[16];
            tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)n0, v);
            if (c < ncol) {
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const int li = n0 + j;
                    if (li < nrows) {
                        const int l = m + par + 2 * li;
                        float *d = A + ((int64_t)l * (l + 1) / 2 + m) * ncol + c;
                        *d = accumulate ? *d + v[j] : v[j];
                    }
                }
            }
        }
    }
    fence_before();
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols_tmem) : "memory");
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

// Synthesis, per block z = (m, parity), ring tile nt and a tile of 128 columns:
//   G[parity][m][r][c] = sum_li lambda[z][li][r] * A[l(li)(l+1)/2 + m][c]
// MMA shape M = 128 (columns), N = NT rings, K = rows li in chunks of KC.
// The A rows are split by the threads; the lambda^T planes come from the
// synthesis table (one bulk copy per chunk).
__global__ void __launch_bounds__(NTHREADS) k_leg_synthesis_tc(const __nv_bfloat16 *__restrict__ lamts,
                                                                const int64_t *__restrict__ lamts_off, int lmax,
                                                                int nrn, int NT, const float *__restrict__ A,
                                                                int64_t ncol, float *__restrict__ G, int *err) {
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
        for (int rr = warp; rr < NT; rr += NTHREADS / 32) {
            const int r = r0 + rr;
            if (r >= nrn) break;
            for (int64_t c = col0 + lane; c < col0 + MTILE && c < ncol; c += 32) Gz[(int64_t)r * ncol + c] = 0.f;
        }
        return;
    }
    const int nK = (nrows + KC - 1) / KC;
    const int ntiles = (nrn + NT - 1) / NT;
    const uint32_t planeA = MTILE * KC * 2;
    const uint32_t planeB = (uint32_t)NT * KC * 2;
    unsigned char *sA = smem;
    unsigned char *sB = smem + 3 * planeA;
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + 3 * planeA + 3 * planeB);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 2);
    const uint32_t ncols_tmem = NT <= 32 ? 32 : (NT <= 64 ? 64 : (NT <= 128 ? 128 : 256));
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(ncols_tmem)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tmem_slot;
    // table block of (z, nt): nK chunks of 3 planes of NT x KC
    const __nv_bfloat16 *Lz = lamts + lamts_off[z] + (int64_t)nt * nK * 3 * NT * KC;
    const uint32_t chunkB = 3u * planeB;
    const uint32_t idesc = idesc_bf16(MTILE, NT);
    const uint32_t sbo = (KC / 8) * 128;
    bool ok = true;
    for (int kc = 0; kc < nK && ok; ++kc) {
        const uint32_t phase = (uint32_t)(kc & 1);
        if (tid == 0) {
            mbar_expect_tx(&bars[0], chunkB);
            bulk_g2s(sB, Lz + (int64_t)kc * 3 * NT * KC, chunkB, &bars[0]);
        }
        const int c = tid;
        const bool cok = col0 + c < ncol;
#pragma unroll 4
        for (int k = 0; k < KC; k += 2) {
            const int li0 = kc * KC + k;
            float v0 = 0.f, v1 = 0.f;
            if (cok) {
                if (li0 < nrows) {
                    const int l = m + par + 2 * li0;
                    v0 = A[((int64_t)l * (l + 1) / 2 + m) * ncol + col0 + c];
                }
                if (li0 + 1 < nrows) {
                    const int l = m + par + 2 * (li0 + 1);
                    v1 = A[((int64_t)l * (l + 1) / 2 + m) * ncol + col0 + c];
                }
            }
            __nv_bfloat16 h0, m0, l0, h1, m1, l1;
            split3(v0, h0, m0, l0);
            split3(v1, h1, m1, l1);
            const uint32_t off = core_off(c, k);
            *reinterpret_cast<__nv_bfloat162 *>(sA + off) = __halves2bfloat162(h0, h1);
            *reinterpret_cast<__nv_bfloat162 *>(sA + planeA + off) = __halves2bfloat162(m0, m1);
            *reinterpret_cast<__nv_bfloat162 *>(sA + 2 * planeA + off) = __halves2bfloat162(l0, l1);
        }
        fence_proxy_async();
        __syncthreads();
        if (tid == 0) {
            if (!mbar_wait(&bars[0], phase)) {
                atomicOr(err, ERR_TC_TIMEOUT);
                ok = false;
            } else {
                fence_after();
                const uint32_t a0 = smem_u32(sA), b0 = smem_u32(sB);
#pragma unroll
                for (int s = 0; s < KC / 16; ++s) {
#pragma unroll
                    for (int q = 0; q < 6; ++q) {
                        const uint64_t ad = smem_desc(a0 + kPairA[q] * planeA + s * 256, 128, sbo);
                        const uint64_t bd = smem_desc(b0 + kPairB[q] * planeB + s * 256, 128, sbo);
                        mma_bf16(tmem, ad, bd, idesc, (kc > 0 || s > 0 || q > 0) ? 1u : 0u);
                    }
                }
                mma_commit(&bars[1]);
            }
        }
        ok = __syncthreads_and(ok);
        if (!ok) break;
        if (!mbar_wait(&bars[1], phase)) {
            atomicOr(err, ERR_TC_TIMEOUT);
            ok = false;
        }
        ok = __syncthreads_and(ok);
    }
    (void)ntiles;
    fence_after();
    if (ok) {
        const int64_t c = col0 + warp * 32 + lane;
        for (int n0 = 0; n0 < NT; n0 += 16) {
            float v[16];
            tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)n0, v);
            if (c < ncol) {
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const int r = r0 + n0 + j;
                    if (r < nrn) Gz[(int64_t)r * ncol + c] = v[j];
                }
            }
        }
    }
    fence_before();
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols_tmem) : "memory");
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

}  // namespace tc

int tc_chunks(const Plan &p) { return (int)((p.nrn + tc::KC - 1) / tc::KC); }

int tc_np_max(const Plan &p) {
    const int nr = p.lmax / 2 + 1;
    return (nr + 15) & ~15;
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

size_t tc_analysis_smem(const Plan &p) {
    return 3 * (size_t)tc::MTILE * tc::KC * 2 + 3 * (size_t)tc_np_max(p) * tc::KC * 2 + 64;
}

void launch_leg_analysis_tc(const Plan &p, const float *F, int64_t ncol, float *A, bool accumulate, cudaStream_t st) {
    const size_t smem = tc_analysis_smem(p);
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(tc::k_leg_analysis_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
        attr = true;
    }
    dim3 grid((unsigned)((ncol + tc::MTILE - 1) / tc::MTILE), 1, (unsigned)(2 * (p.lmax + 1)));
    tc::k_leg_analysis_tc<<<grid, tc::NTHREADS, smem, st>>>((const __nv_bfloat16 *)p.d_lamtc, p.d_lamtc_off, p.lmax,
                                                           (int)p.nrn, tc_chunks(p), F, ncol, A, accumulate ? 1 : 0,
                                                           tc_np_max(p), p.d_err);
    note_launch();
}

}  // namespace sfb

namespace sfb {

int tc_synth_nt(const Plan &p) {
    const int nrn = (int)p.nrn;
    const int nt16 = (nrn + 15) & ~15;
    return nt16 < 256 ? nt16 : 256;
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

void launch_leg_synthesis_tc(const Plan &p, const float *A, int64_t ncol, float *G, cudaStream_t st) {
    const int NT = tc_synth_nt(p);
    const size_t smem = 3 * (size_t)tc::MTILE * tc::KC * 2 + 3 * (size_t)NT * tc::KC * 2 + 64;
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(tc::k_leg_synthesis_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
        attr = true;
    }
    dim3 grid((unsigned)((ncol + tc::MTILE - 1) / tc::MTILE), (unsigned)((p.nrn + NT - 1) / NT),
              (unsigned)(2 * (p.lmax + 1)));
    tc::k_leg_synthesis_tc<<<grid, tc::NTHREADS, smem, st>>>((const __nv_bfloat16 *)p.d_lamts, p.d_lamts_off, p.lmax,
                                                            (int)p.nrn, NT, A, ncol, G, p.d_err);
    note_launch();
}

}  // namespace sfb
