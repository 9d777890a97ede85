// Legendre contractions on the 5th-generation tensor cores (tcgen05), used
// by the mixed-precision transform.
//
// Analysis, per block z = (m, parity) and a tile of 128 columns c (re/im of
// the maps):
//   A[l(li)(l+1)/2 + m][c] (+)= sum_r F[parity][m][r][c] * lambda[z][li][r]
// MMA shape M = 128 (columns c), N = rows li padded to 16 (<= 128 per tile),
// K = rings in chunks of KC.
// Synthesis, per block z, ring tile and column tile:
//   G[parity][m][r][c] = sum_li lambda[z][li][r] * A[l(li)(l+1)/2 + m][c]
// MMA shape M = 128 (columns), N = rings (<= 128 per tile), K = rows li.
//
// Error-free splitting (block-floating-point slicing, Ozaki, Ogita, Oishi,
// Rump, Numer. Algorithms 59, 2012): every operand value is written as four
// BF16 slices on a scale common to its whole K range - per lambda row (plan
// tables), per column of F or A (a max pass over the CTA's K range) - with
// 8-bit slice steps, so each operand is represented to 2^-31 (A: 7-bit
// leading slice) or 2^-32 (lambda, F: 8-bit leading slice) of its scale.  The
// products of slice level v = s_a + s_b (v = 0..3; ten products) are integer
// multiples of one unit per accumulator entry and each level has its own FP32
// accumulator in TMEM; the level-0 sums stay within 2^24 units for K <= 1024
// (ring pairs) and K <= 512 (rows), so they are exact whatever the tensor
// cores' accumulation order or rounding, and the level-v sums (v >= 1) carry
// 2^(-8 v) of the leading one, so a rounding there stays below 2^-32 of it.
// Levels >= 4 (below 2^-32 of the leading products) are dropped.  The
// epilogue adds the four levels with one significant rounding.
//
// The F (analysis) and A (synthesis) tiles are sliced by the CTA's threads
// into four K-major BF16 planes in shared memory; the lambda planes come
// pre-sliced from the plan's tables by bulk copy (cp.async.bulk, TMA engine).
// Two shared-memory stages and N <= 64 per CTA (256 TMEM columns), so two
// CTAs share an SM: the next chunk's lambda planes and operand values are
// fetched while the tensor cores work on the current one, and the other
// CTA covers the latencies.  The per-column scales of F come from a
// separate bandwidth-bound pass (k_colmax).  The
// analysis keeps a double-float copy of A (float2) beside the FP64 one, which
// the synthesis slices without FP64 arithmetic.
//
// Shared-memory operand layout (no swizzle, K-major): 8x8 "core matrices" of
// 128 contiguous bytes (8 rows of 8 bf16); core (g, kk) of a plane sits at
// ((g * KC/8) + kk) * 128 bytes, so the descriptor's leading byte offset
// (next core along K) is 128 and the stride byte offset (next 8-row group)
// is KC/8 * 128.
//
// Every wait on an mbarrier is bounded; on timeout the CTA records
// ERR_TC_TIMEOUT in the plan's error word, waits (bounded) for its MMAs,
// releases its TMEM and returns.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>

#include "sfb_internal.h"
#include "tc_common.cuh"

namespace sfb {
namespace tc {

constexpr int KC = 16;          // K elements per chunk (one MMA K step)
constexpr int MTILE = 128;      // columns per CTA (MMA M)
constexpr int NMAX = 64;        // MMA N per CTA: lambda rows (analysis) or rings (synthesis)
constexpr int NPROD = 256;      // producer threads: two per operand row (warps 0-7)
constexpr int NTH = NPROD + 32; // + the MMA warp (warp 8)
constexpr int NSTAGE = 4;
constexpr uint32_t PLANE_A = MTILE * KC * 2;          // bytes of one operand-A plane
constexpr uint32_t PLANE_B = NMAX * KC * 2;           // bytes of one lambda plane (<= NMAX rows)
constexpr uint32_t STAGE_BYTES = 4 * PLANE_A + 4 * PLANE_B;
constexpr uint32_t TMEM_COLS = 4 * NMAX;             // four level accumulators
constexpr size_t LEG_SMEM = NSTAGE * (size_t)STAGE_BYTES + 128;  // two CTAs per SM

// byte offset of element (row, k) in a K-major no-swizzle plane with KC columns
__device__ __forceinline__ uint32_t core_off(int row, int k) {
    return (uint32_t)((((row >> 3) * (KC / 8) + (k >> 3)) << 7) + ((row & 7) << 4) + ((k & 7) << 1));
}

__device__ __forceinline__ int rows_of(int m, int par, int lmax) {
    return (m + par <= lmax) ? (lmax - m - par) / 2 + 1 : 0;
}

__device__ __forceinline__ int pad16(int n) { return (n + 15) & ~15; }

__device__ __forceinline__ void st_v4(unsigned char *p, const uint32_t (&v)[4]) {
    *reinterpret_cast<uint4 *>(p) = make_uint4(v[0], v[1], v[2], v[3]);
}

// Shared state of the level kernels: NSTAGE stages of (A planes, B planes)
// and the barriers of the producer / MMA pipeline: full_a[s] (every producer
// warp wrote its slices: one arrival per warp after __syncwarp), full_b[s] (lambda planes landed), empty[s]
// (the MMAs of the stage completed), done (all MMAs completed).
struct LvlSmem {
    unsigned char *base;
    uint64_t *full_a, *full_b, *empty, *done;
    uint32_t *slot;
    int *bad;
    __device__ __forceinline__ unsigned char *stage(int s) const { return base + s * STAGE_BYTES; }
};

__device__ __forceinline__ LvlSmem lvl_smem(unsigned char *base) {
    LvlSmem c;
    c.base = base;
    c.full_a = reinterpret_cast<uint64_t *>(base + NSTAGE * STAGE_BYTES);
    c.full_b = c.full_a + NSTAGE;
    c.empty = c.full_b + NSTAGE;
    c.done = c.empty + NSTAGE;
    c.slot = reinterpret_cast<uint32_t *>(c.done + 1);
    c.bad = reinterpret_cast<int *>(c.slot + 1);
    return c;
}

__device__ __forceinline__ uint32_t lvl_setup(LvlSmem &c) {
    if ((threadIdx.x >> 5) == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(c.slot)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (threadIdx.x == 0) {
        for (int i = 0; i < NSTAGE; ++i) {
            mbar_init(&c.full_a[i], NPROD / 32);
            mbar_init(&c.full_b[i], 1);
            mbar_init(&c.empty[i], 1);
        }
        mbar_init(c.done, 1);
        *c.bad = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    return *c.slot;
}

__device__ __forceinline__ void lvl_teardown(uint32_t tmem) {
    fence_before();
    __syncthreads();
    if ((threadIdx.x >> 5) == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
}

// The ten level products of one K chunk (one K step of 16) as six MMAs
// (tc_common.cuh): level v goes to TMEM columns [LS v, LS v + LS), LS = the
// MMA's N (lambda rows or rings of this CTA).
__device__ __forceinline__ void lvl_mma(uint32_t tmem, uint32_t a0, uint32_t b0, uint32_t planeB, int LS,
                                        bool first_chunk) {
    const uint32_t sbo = (KC / 8) * 128;
    const uint32_t id1 = idesc_bf16(MTILE, LS), id2 = idesc_bf16(MTILE, 2 * LS);
#pragma unroll
    for (int q = 0; q < NMERGED; ++q) {
        const uint64_t ad = smem_desc(a0 + mg_a(q) * PLANE_A, 128, sbo);
        const uint64_t bd = smem_desc(b0 + mg_b(q) * planeB, 128, sbo);
        const uint32_t acc = (first_chunk && mg_first(q)) ? 0u : 1u;
        mma_bf16(tmem + (uint32_t)LS * (uint32_t)mg_lvl(q), ad, bd, mg_two(q) ? id2 : id1, acc);
    }
}

// Sum of the four level accumulators of one entry as a double-float (hi, lo):
// (s, e) = TwoSum(L0, L1), then lo = e + (L2 + L3), renormalised.
__device__ __forceinline__ void lvl_sum(float L0, float L1, float L2, float L3, float &hi, float &lo) {
    const float s = L0 + L1;
    const float z = s - L0;
    const float e = (L0 - (s - z)) + (L1 - z);
    const float t = e + (L2 + L3);
    hi = s + t;
    lo = t - (hi - s);
}

// Chunk kc lives in stage kc % NSTAGE, the (kc / NSTAGE)-th use of that stage.
__device__ __forceinline__ uint32_t ph_of(int kc) { return (uint32_t)((kc / NSTAGE) & 1); }

// MMA warp (lane 0 issues): for every chunk wait for its A slices and lambda
// planes, issue the ten products, release the stage; finally commit `done`.
// Returns the number of chunks issued.
__device__ __forceinline__ int lvl_mma_loop(const LvlSmem &cs, uint32_t tmem, int nch, uint32_t planeB, int LS) {
    int issued = 0;
    for (int kc = 0; kc < nch; ++kc) {
        const int s = kc % NSTAGE;
        if (*(volatile int *)cs.bad) break;
        if (!mbar_wait(&cs.full_a[s], ph_of(kc)) || !mbar_wait(&cs.full_b[s], ph_of(kc))) {
            atomicExch(cs.bad, 1);
            break;
        }
        fence_after();
        const uint32_t sa = smem_u32(cs.stage(s));
        lvl_mma(tmem, sa, sa + 4 * PLANE_A, planeB, LS, kc == 0);
        mma_commit(&cs.empty[s]);
        ++issued;
    }
    mma_commit(cs.done);          // arrives once every MMA issued above has completed
    return issued;
}

// Producer side of one chunk: wait until the stage is free (its previous
// MMAs completed), optionally start the lambda copy, write the A slices and
// arrive on full_a.  False when a wait expired.
__device__ __forceinline__ bool lvl_stage_free(const LvlSmem &cs, int kc) {
    if (kc < NSTAGE) return true;
    if (*(volatile int *)cs.bad) return false;
    if (!mbar_wait(&cs.empty[kc % NSTAGE], (uint32_t)(((kc / NSTAGE) - 1) & 1))) {
        atomicExch(cs.bad, 1);
        return false;
    }
    return true;
}

// Per (block z, column c): E with max_r |F[parity][m][r][c]| < 2^E, raised by
// ceil(log2 nrn) - 10 for more than 1024 ring pairs, so that the exact level
// sums (8-bit leading slices of F and lambda, at most 2^14 units a product)
// stay within 2^24 units.
// (nzr: F is zero outside the ring pairs [nzr[0], nzr[1]], which are the only ones read)
__global__ void __launch_bounds__(256) k_colmax(const float2 *__restrict__ F, int64_t ncol, int lmax, int nrn,
                                                int *__restrict__ Ecol, const int *__restrict__ nzr,
                                                const int2 *__restrict__ live, int ntile) {
    const int z = blockIdx.y;
    const int m = z >> 1, par = z & 1;
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncol) return;
    const float2 *Fz = F + ((int64_t)(par * (lmax + 1) + m) * nrn) * ncol + c;
    float m0 = 0.f, m1 = 0.f, m2 = 0.f, m3 = 0.f;
    int r = 0, r1 = nrn;
    if (nzr) {
        r = nzr[0];
        r1 = min(nrn, nzr[1] + 1);
    }
    if (live) {          // only the rings of the analysis's live chunks are read (and written)
        int lo = 0x7fffffff, hi = -1;
        for (int t = 0; t < ntile; ++t) {
            const int2 lv = live[(int64_t)z * ntile + t];
            lo = min(lo, lv.x);
            hi = max(hi, lv.y);
        }
        r = max(r, lo * KC);
        r1 = min(r1, (hi + 1) * KC);
    }
    for (; r + 3 < r1; r += 4) {
        m0 = fmaxf(m0, fabsf(Fz[(int64_t)r * ncol].x));
        m1 = fmaxf(m1, fabsf(Fz[(int64_t)(r + 1) * ncol].x));
        m2 = fmaxf(m2, fabsf(Fz[(int64_t)(r + 2) * ncol].x));
        m3 = fmaxf(m3, fabsf(Fz[(int64_t)(r + 3) * ncol].x));
    }
    for (; r < r1; ++r) m0 = fmaxf(m0, fabsf(Fz[(int64_t)r * ncol].x));
    const int lg = 32 - __clz(nrn > 1 ? nrn - 1 : 1);
    Ecol[(int64_t)z * ncol + c] = max(-90, min(scale_exp(fmaxf(fmaxf(m0, m1), fmaxf(m2, m3))) + max(0, lg - 10), 100));
}

// Analysis: grid (column tiles, row tiles of NMAX, blocks z); warps 0-7
// produce (thread: column c, half kh of each chunk), warp 8 issues the MMAs.
// Rings r >= rlim count as zero (the sum over the first rlim rings only).
__global__ void __launch_bounds__(NTH, 2) k_leg_analysis_tc(const __nv_bfloat16 *__restrict__ lamtc,
                                                            const int64_t *__restrict__ lamtc_off, int lmax, int nrn,
                                                            int nchunks, int rlim, const float2 *__restrict__ F,
                                                            int64_t ncol, const int *__restrict__ Ecol,
                                                            double *__restrict__ A, float2 *__restrict__ Adf,
                                                            int accumulate, int *__restrict__ Eout,
                                                            const int *__restrict__ nzr,
                                                            const int2 *__restrict__ live, int *err) {
    extern __shared__ __align__(1024) unsigned char smem[];
    const int z = blockIdx.z;
    const int m = z >> 1, par = z & 1;
    const int nrows = rows_of(m, par, lmax);
    const int NP = pad16(nrows);
    const int row0 = blockIdx.y * NMAX;
    if (row0 >= NP) return;
    const int NPc = min(NMAX, NP - row0);
    const int64_t col0 = (int64_t)blockIdx.x * MTILE;
    const int tid = threadIdx.x, warp = tid >> 5;
    const int c = tid & (MTILE - 1), kh = (tid >> 7) & 1;
    const bool prod = tid < NPROD;
    const bool cok = prod && col0 + c < ncol;
    // Chunk range [lo, hi]: nzr - the ring pairs outside [nzr[0], nzr[1]] carry zero spectra; live -
    // the chunks of this row tile whose lambda slices are not all zero.  Products with the other
    // chunks are exactly zero.  An empty range adds nothing (accumulate: the CTA returns) or gives
    // zero coefficients (no MMA; the epilogue writes zeros).
    int lo = 0, hi = nchunks - 1;
    if (nzr) {
        const int a = nzr[0], b = nzr[1];
        if (b >= a) {
            lo = max(lo, a / KC);
            hi = min(hi, b / KC);
        } else {
            hi = lo - 1;
        }
    }
    if (live) {
        const int2 lv = live[(int64_t)z * gridDim.y + blockIdx.y];
        lo = max(lo, lv.x);
        hi = min(hi, lv.y);
    }
    if (hi < lo && accumulate) return;
    const int kc0 = hi < lo ? 0 : lo;
    nchunks = hi < lo ? 0 : hi - lo + 1;
    const float2 *Fz = F + ((int64_t)(par * (lmax + 1) + m) * nrn + (int64_t)kc0 * KC) * ncol + col0 + c;
    const __nv_bfloat16 *Lz = lamtc + lamtc_off[z] + (int64_t)kc0 * 4 * pad16(rows_of(m, par, lmax)) * KC;
    rlim -= kc0 * KC;
    const uint32_t planeB = (uint32_t)NPc * KC * 2;
    LvlSmem cs = lvl_smem(smem);
    float C[4];
    {
        // a column with no non-zero value anywhere keeps the preset (below any exponent): any scale
        // slices its zeros exactly
        const int ev = cok ? Ecol[(int64_t)z * ncol + col0 + c] : 0;
        slice_consts8(ev < -1000 ? 0 : ev, C);
    }
    const uint32_t tmem = lvl_setup(cs);
    const int LS = NPc;                         // MMA N and TMEM level stride

    if (!prod) {
        if ((tid & 31) == 0) {
            const int issued = lvl_mma_loop(cs, tmem, nchunks, planeB, LS);
            if (issued != nchunks) atomicExch(cs.bad, 1);
        }
    } else {
        float2 pre[2][8];         // this thread's 8 double-float ring values of chunks kc, kc + 1
        auto loadA = [&](int kc, float2 (&buf)[8]) {
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int r = kc * KC + 8 * kh + j;
                buf[j] = (cok && r < rlim) ? Fz[(int64_t)r * ncol] : make_float2(0.f, 0.f);
            }
        };
        auto chunk = [&](int kc, float2 (&cur)[8]) -> bool {
            const int s = kc % NSTAGE;
            if (!lvl_stage_free(cs, kc)) return false;
            unsigned char *sa = cs.stage(s);
            if (tid == 0) {
                mbar_expect_tx(&cs.full_b[s], 4 * planeB);
                const int64_t chunk_elems = 4LL * NP * KC;
                for (int pl = 0; pl < 4; ++pl)
                    bulk_g2s(sa + 4 * PLANE_A + pl * planeB,
                             Lz + kc * chunk_elems + (int64_t)pl * NP * KC + (int64_t)row0 * KC, planeB,
                             &cs.full_b[s]);
            }
            uint32_t w[4][4];
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                uint32_t v[4];
                slice_pair_df(cur[2 * t].x, cur[2 * t].y, cur[2 * t + 1].x, cur[2 * t + 1].y, C, v);
#pragma unroll
                for (int q = 0; q < 4; ++q) w[q][t] = v[q];
            }
            const uint32_t off = core_off(c, 8 * kh);
#pragma unroll
            for (int q = 0; q < 4; ++q) st_v4(sa + q * PLANE_A + off, w[q]);
            if (kc + 2 < nchunks) loadA(kc + 2, cur);
            fence_proxy_async();
            __syncwarp();
            if ((tid & 31) == 0) mbar_arrive(&cs.full_a[s]);       // one arrival per producer warp
            return true;
        };
#pragma unroll
        for (int q = 0; q < 2; ++q)
            if (q < nchunks) loadA(q, pre[q]);
        for (int kc = 0; kc < nchunks; kc += 2) {
            if (!chunk(kc, pre[0])) break;
            if (kc + 1 < nchunks && !chunk(kc + 1, pre[1])) break;
        }
    }
    // every thread: wait for all MMAs, then the epilogue
    bool ok = mbar_wait(cs.done, 0);
    fence_after();
    ok = __syncthreads_and(ok) && !*(volatile int *)cs.bad;
    if (!ok) {
        if (tid == 0) atomicOr(err, ERR_TC_TIMEOUT);
    } else if (prod) {
        // warp w reads TMEM lanes 32 (w % 4).. (columns) and rows li in [32 (w / 4), +32), eight rows at a
        // time: the eight rows' old values are loaded together (no dependent round trips)
        const int lq = warp & 3, hg = warp >> 2;
        const uint32_t lane_base = (uint32_t)(lq * 32) << 16;
        const int64_t cc = col0 + lq * 32 + (tid & 31);
        float mx = 0.f;
        for (int g = 0; g < 4; ++g) {
            const int i0 = 32 * hg + 8 * g;
            if (i0 >= NPc) break;                           // warp-uniform
            float v0[8], v1[8], v2[8], v3[8];
            tmem_ld8(tmem + lane_base + (uint32_t)i0, v0);
            tmem_ld8(tmem + lane_base + (uint32_t)(LS + i0), v1);
            tmem_ld8(tmem + lane_base + (uint32_t)(2 * LS + i0), v2);
            tmem_ld8(tmem + lane_base + (uint32_t)(3 * LS + i0), v3);
            if (nchunks == 0) {           // no MMA wrote the accumulators: the sums are zero
#pragma unroll
                for (int i = 0; i < 8; ++i) v0[i] = v1[i] = v2[i] = v3[i] = 0.f;
            }
            if (cc < ncol) {
                auto off = [&](int i) {
                    const int l = m + par + 2 * (row0 + i0 + i);
                    return ((int64_t)l * (l + 1) / 2 + m) * ncol + cc;
                };
                double aold[8];
                float2 dold[8];
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    aold[i] = 0.0;
                    dold[i] = make_float2(0.f, 0.f);
                    if (accumulate && row0 + i0 + i < nrows) {
                        const int64_t o = off(i);
                        if (A) aold[i] = A[o];
                        dold[i] = Adf[o];
                    }
                }
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    if (row0 + i0 + i >= nrows) continue;
                    const int64_t o = off(i);
                    float hi, lo;
                    lvl_sum(v0[i], v1[i], v2[i], v3[i], hi, lo);
                    // double-float accumulation of (hi, lo) into the old value (zero without accumulate)
                    const float2 d = dold[i];
                    const float s = d.x + hi;
                    const float zz = s - d.x;
                    const float e = ((d.x - (s - zz)) + (hi - zz)) + (d.y + lo);
                    const float h2 = s + e;
                    Adf[o] = make_float2(h2, e - (h2 - s));
                    if (A) A[o] = aold[i] + ((double)hi + (double)lo);
                    mx = fmaxf(mx, fabsf(h2));
                }
            }
        }
        // column exponent of the new coefficients (the synthesis-side slicing scale)
        // (threads without a row in range, or with only zeros, leave the column's preset value)
        if (Eout && cc < ncol && mx > 0.f) atomicMax(Eout + (int64_t)z * ncol + cc, scale_exp(mx));
    }
    lvl_teardown(tmem);
}

// Synthesis: grid (column tiles, ring tiles of NT <= NMAX, blocks z); warps
// 0-7 produce, warp 8 issues the MMAs.
//
// Update mode (Adfnew != nullptr): the table holds D = M - I, M the Gram
// matrices of the alias-free rings; "rings" r are output rows li (nrn = rows of
// the largest block), and the epilogue writes, instead of G,
//   Anew[l(r)] = A0[l(r)] - sum_li D[r][li] Acur[l(li)]
// (= Acur + (A0 - M Acur)) in double-float and, when Anew is given, in FP64.
// |D| is the polar rings' share of the quadrature, so the product's FP32
// accumulation error is that share of |Acur|, not all of it.
__global__ void __launch_bounds__(NTH, 2) k_leg_synthesis_tc(const __nv_bfloat16 *__restrict__ lamts,
                                                             const int64_t *__restrict__ lamts_off, int lmax, int nrn,
                                                             int NT, const float2 *__restrict__ Adf, int64_t ncol,
                                                             float *__restrict__ G, const double *__restrict__ Acur,
                                                             const float2 *__restrict__ A0, double *__restrict__ Anew,
                                                             float2 *__restrict__ Adfnew, const int *__restrict__ Ein,
                                                             int *__restrict__ Eout, const int2 *__restrict__ live,
                                                             int *err) {
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ float red[2][MTILE];
    const int z = blockIdx.z;
    const int m = z >> 1, par = z & 1;
    const int nrows = rows_of(m, par, lmax);
    const int nt = blockIdx.y;
    const int r0 = nt * NT;
    const int64_t col0 = (int64_t)blockIdx.x * MTILE;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const bool upd = Adfnew != nullptr;
    if (upd && r0 >= nrows) return;          // no output row of this block in the tile
    float *Gz = upd ? nullptr : G + ((int64_t)(par * (lmax + 1) + m) * nrn) * ncol;
    // live: the row chunks [lv.x, lv.y] of this ring tile whose lambda slices are not all zero (the
    // products with the others are exactly zero); none - the tile's G is zero
    int k0 = 0, nK = (nrows + KC - 1) / KC;
    if (live && nrows > 0) {
        const int2 lv = live[(int64_t)z * ((nrn + NT - 1) / NT) + nt];      // the table's ring tiles
        k0 = lv.x;
        nK = lv.y >= lv.x ? lv.y - lv.x + 1 : 0;
    }
    if (nrows == 0 || nK == 0) {      // no l for this (m, parity), or no live chunk: the tile is zero
        for (int rr = warp; rr < NT; rr += NTH / 32) {
            const int r = r0 + rr;
            if (r >= nrn) break;
            for (int64_t cc = col0 + lane; cc < col0 + MTILE && cc < ncol; cc += 32) Gz[(int64_t)r * ncol + cc] = 0.f;
        }
        return;
    }
    const int c = tid & (MTILE - 1), kh = (tid >> 7) & 1;
    const bool prod = tid < NPROD;
    const bool cok = prod && col0 + c < ncol;
    const uint32_t planeB = (uint32_t)NT * KC * 2;
    const __nv_bfloat16 *Lz = lamts + lamts_off[z] + ((int64_t)nt * ((nrows + KC - 1) / KC) + k0) * 4 * NT * KC;
    LvlSmem cs = lvl_smem(smem);
    auto aval = [&](int li) -> float2 {
        if (!cok || li >= nrows) return make_float2(0.f, 0.f);
        const int l = m + par + 2 * li;
        return Adf[((int64_t)l * (l + 1) / 2 + m) * ncol + col0 + c];
    };
    // column scale over the rows (|hi + lo| < 2^E: hi is an FP32 value below 2^E, |lo| <= ulp(hi)/2):
    // given by the kernel that wrote the coefficients (Ein), or a pass over them here
    if (!Ein) {
        float mx = 0.f;
        for (int li = kh; li < nrows; li += 2) mx = fmaxf(mx, fabsf(aval(li).x));
        if (prod) red[kh][c] = mx;
    }
    const uint32_t tmem = lvl_setup(cs);      // includes a __syncthreads
    float C[4];
    int Ecl = 0;
    if (Ein) {
        // an all-zero column keeps the preset (below any exponent): any scale slices zeros exactly
        const int ev = cok ? Ein[(int64_t)z * ncol + col0 + c] : 0;
        Ecl = ev < -1000 ? 0 : ev;
    } else {
        Ecl = scale_exp(fmaxf(red[0][c], red[1][c]));
    }
    slice_consts(Ecl, C);
    const int LS = NT;                          // MMA N and TMEM level stride

    if (!prod) {
        if (lane == 0) {
            const int issued = lvl_mma_loop(cs, tmem, nK, planeB, LS);
            if (issued != nK) atomicExch(cs.bad, 1);
        }
    } else {
        float2 pre[2][8];
        auto loadA = [&](int kc, float2 (&buf)[8]) {
#pragma unroll
            for (int j = 0; j < 8; ++j) buf[j] = aval((k0 + kc) * KC + 8 * kh + j);
        };
        auto chunk = [&](int kc, float2 (&cur)[8]) -> bool {
            const int s = kc % NSTAGE;
            if (!lvl_stage_free(cs, kc)) return false;
            unsigned char *sa = cs.stage(s);
            if (tid == 0) {
                mbar_expect_tx(&cs.full_b[s], 4 * planeB);
                bulk_g2s(sa + 4 * PLANE_A, Lz + (int64_t)kc * 4 * NT * KC, 4 * planeB, &cs.full_b[s]);
            }
            uint32_t w[4][4];
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                uint32_t v[4];
                slice_pair_df(cur[2 * t].x, cur[2 * t].y, cur[2 * t + 1].x, cur[2 * t + 1].y, C, v);
#pragma unroll
                for (int q = 0; q < 4; ++q) w[q][t] = v[q];
            }
            const uint32_t off = core_off(c, 8 * kh);
#pragma unroll
            for (int q = 0; q < 4; ++q) st_v4(sa + q * PLANE_A + off, w[q]);
            if (kc + 2 < nK) loadA(kc + 2, cur);
            fence_proxy_async();
            __syncwarp();
            if ((tid & 31) == 0) mbar_arrive(&cs.full_a[s]);       // one arrival per producer warp
            return true;
        };
        loadA(0, pre[0]);
        if (nK > 1) loadA(1, pre[1]);
        for (int kc = 0; kc < nK; kc += 2) {
            if (!chunk(kc, pre[0])) break;
            if (kc + 1 < nK && !chunk(kc + 1, pre[1])) break;
        }
    }
    bool ok = mbar_wait(cs.done, 0);
    fence_after();
    ok = __syncthreads_and(ok) && !*(volatile int *)cs.bad;
    if (!ok) {
        if (tid == 0) atomicOr(err, ERR_TC_TIMEOUT);
    } else if (prod) {
        // warp w reads TMEM lanes 32 (w % 4).. (columns) and rings [32 (w / 4), +32) of the tile
        const int lq = warp & 3, hg = warp >> 2;
        const uint32_t lane_base = (uint32_t)(lq * 32) << 16;
        const int64_t cc = col0 + lq * 32 + lane;
        float umx = 0.f;          // update mode: largest new |coefficient| of this column
        for (int g = 0; g < 4; ++g) {
            const int i0 = 32 * hg + 8 * g;
            if (i0 >= NT) break;                            // warp-uniform
            float v0[8], v1[8], v2[8], v3[8];
            tmem_ld8(tmem + lane_base + (uint32_t)i0, v0);
            tmem_ld8(tmem + lane_base + (uint32_t)(LS + i0), v1);
            tmem_ld8(tmem + lane_base + (uint32_t)(2 * LS + i0), v2);
            tmem_ld8(tmem + lane_base + (uint32_t)(3 * LS + i0), v3);
            if (cc < ncol && !upd) {
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    const int r = r0 + i0 + i;
                    if (r >= nrn) break;
                    float hi, lo;
                    lvl_sum(v0[i], v1[i], v2[i], v3[i], hi, lo);
                    Gz[(int64_t)r * ncol + cc] = hi;
                }
            } else if (cc < ncol) {
                // the eight rows' old values are loaded together (no dependent round trips)
                auto off = [&](int i) {
                    const int l = m + par + 2 * (r0 + i0 + i);
                    return ((int64_t)l * (l + 1) / 2 + m) * ncol + cc;
                };
                float2 a0[8];
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    a0[i] = make_float2(0.f, 0.f);
                    if (r0 + i0 + i < nrows) a0[i] = A0[off(i)];
                }
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    if (r0 + i0 + i >= nrows) continue;
                    const int64_t o = off(i);
                    float hi, lo;
                    lvl_sum(v0[i], v1[i], v2[i], v3[i], hi, lo);
                    // A0 - (hi, lo) in double-float (TwoSum, renormalised)
                    const float s = a0[i].x - hi, z2 = s - a0[i].x;
                    const float e = ((a0[i].x - (s - z2)) + (-hi - z2)) + (a0[i].y - lo);
                    const float nh = s + e, nl = e - (nh - s);
                    Adfnew[o] = make_float2(nh, nl);
                    if (Anew) Anew[o] = (double)nh + (double)nl;
                    umx = fmaxf(umx, fabsf(nh));
                }
            }
        }
        if (upd && Eout && cc < ncol && umx > 0.f) atomicMax(Eout + (int64_t)z * ncol + cc, scale_exp(umx));
    }
    lvl_teardown(tmem);
}

// Row scales of the lambda tables.  Analysis: per (z, li) over the rings;
// synthesis: per (z, ring) over the rows.  E with max |lambda| < 2^E.
__global__ void k_lam_rowexp(const double *__restrict__ lam, const int64_t *lam_off, int lmax, int nrn, int *Ea,
                             int *Es) {
    const int z = blockIdx.y;
    const int m = z >> 1, par = z & 1;
    const int nrows = rows_of(m, par, lmax);
    const double *L = lam + lam_off[z];
    const int64_t rbase = lam_off[z] / nrn;            // first row of block z in the table
    const int lane = threadIdx.x & 31;
    const int nw = blockDim.x >> 5;
    for (int li = blockIdx.x * nw + (threadIdx.x >> 5); li < nrows; li += gridDim.x * nw) {
        double mx = 0.0;
        for (int r = lane; r < nrn; r += 32) mx = fmax(mx, fabs(L[(int64_t)li * nrn + r]));
        for (int off = 16; off > 0; off >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, off));
        if (lane == 0) Ea[rbase + li] = (mx > 0.0 && isfinite(mx)) ? ilogb(mx) + 1 : 0;
    }
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nrn; r += gridDim.x * blockDim.x) {
        double mx = 0.0;
        for (int li = 0; li < nrows; ++li) mx = fmax(mx, fabs(L[(int64_t)li * nrn + r]));
        Es[(int64_t)z * nrn + r] = (mx > 0.0 && isfinite(mx)) ? ilogb(mx) + 1 : 0;
    }
}

// four BF16 slices of v on the scale 2^E: b_k 2^(E - 7 - 8k), |b_k| <= 128
__device__ __forceinline__ void slices4(double v, int E, __nv_bfloat16 (&o)[4]) {
    double y = ldexp(v, 7 - E);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const double a = rint(y);
        y = (y - a) * 256.0;
        o[k] = __double2bfloat16(ldexp(a, E - 7 - 8 * k));      // at most 8 significant bits: exact
    }
}

// Analysis table: block z, chunk kc, plane q, row li < NP, ring k < KC in the
// core-matrix layout (zero padding), sliced on the row scale Ea.
__global__ void k_build_lamtc(const double *__restrict__ lam, const int64_t *lam_off, int lmax, int nrn, int nchunks,
                              const int *__restrict__ Ea, const int64_t *lamtc_off, __nv_bfloat16 *lamtc) {
    const int z = blockIdx.y;
    const int m = z >> 1, par = z & 1;
    const int nrows = rows_of(m, par, lmax);
    if (nrows == 0) return;
    const int NP = pad16(nrows);
    const int64_t rbase = lam_off[z] / nrn;
    const int64_t total = (int64_t)NP * nchunks * KC;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int li = (int)(idx / ((int64_t)nchunks * KC));
        const int rr = (int)(idx - (int64_t)li * nchunks * KC);
        const int kc = rr / KC, k = rr % KC;
        double v = 0.0;
        int E = 0;
        if (li < nrows && rr < nrn) {
            v = lam[lam_off[z] + (int64_t)li * nrn + rr];
            E = Ea[rbase + li];
        }
        __nv_bfloat16 o[4];
        slices4(v, E, o);
        const int64_t base = lamtc_off[z] + (int64_t)kc * 4 * NP * KC;
        const int64_t e = core_off(li, k) >> 1;
#pragma unroll
        for (int q = 0; q < 4; ++q) lamtc[base + (int64_t)q * NP * KC + e] = o[q];
    }
}

// Synthesis table: block z, ring tile nt, chunk kc, plane q, ring rr < NT,
// row k < KC in the core-matrix layout (N = rings, K = rows li), sliced on
// the ring scale Es.
__global__ void k_build_lamts(const double *__restrict__ lam, const int64_t *lam_off, int lmax, int nrn, int NT,
                              const int *__restrict__ Es, const int64_t *lamts_off, __nv_bfloat16 *lamts) {
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
        int E = 0;
        if (r < nrn && li < nrows) {
            v = lam[lam_off[z] + (int64_t)li * nrn + r];
            E = Es[(int64_t)z * nrn + r];
        }
        __nv_bfloat16 o[4];
        slices4(v, E, o);
        const int64_t plane = (int64_t)NT * KC;
        const int64_t base = lamts_off[z] + ((int64_t)nt * nK + kc) * 4 * plane;
        const int64_t e = core_off(rr, k) >> 1;
#pragma unroll
        for (int q = 0; q < 4; ++q) lamts[base + q * plane + e] = o[q];
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

// offsets (in bf16 elements) of every block of the analysis table; returns the total
int64_t tc_table_offsets(const Plan &p, std::vector<int64_t> &off) {
    const int nch = tc_chunks(p);
    off.assign(2 * (p.lmax + 1) + 1, 0);
    int64_t o = 0;
    for (int z = 0; z < 2 * (p.lmax + 1); ++z) {
        const int m = z >> 1, par = z & 1;
        const int nrows = (m + par <= p.lmax) ? (p.lmax - m - par) / 2 + 1 : 0;
        off[z] = o;
        if (nrows > 0) o += 4LL * ((nrows + 15) & ~15) * nch * tc::KC;
    }
    off[2 * (p.lmax + 1)] = o;
    return o;
}

void launch_build_lamtc(const Plan &p, const int *Ea, const int *Es, cudaStream_t st) {
    {
        dim3 grid(8, (unsigned)(2 * (p.lmax + 1)));
        tc::k_lam_rowexp<<<grid, 256, 0, st>>>(p.d_lam, p.d_lam_off, p.lmax, (int)p.nrn, const_cast<int *>(Ea),
                                               const_cast<int *>(Es));
        note_launch();
    }
    dim3 grid(64, (unsigned)(2 * (p.lmax + 1)));
    tc::k_build_lamtc<<<grid, 256, 0, st>>>(p.d_lam, p.d_lam_off, p.lmax, (int)p.nrn, tc_chunks(p), Ea,
                                            p.d_lamtc_off, (__nv_bfloat16 *)p.d_lamtc);
    note_launch();
}

void launch_leg_analysis_tc(const Plan &p, const float2 *F, int64_t ncol, double *A, float2 *Adf, int *Ecol,
                            bool accumulate, cudaStream_t st, bool scales_ready, int rlim, int *Eout,
                            const int *nzr) {
    if (rlim < 0 || rlim > p.nrn) rlim = (int)p.nrn;
    if (!scales_ready) {
        dim3 grid((unsigned)((ncol + 255) / 256), (unsigned)(2 * (p.lmax + 1)));
        tc::k_colmax<<<grid, 256, 0, st>>>(F, ncol, p.lmax, (int)p.nrn, Ecol, nzr, p.d_lamtc_live,
                                           (tc_np_max(p) + tc::NMAX - 1) / tc::NMAX);
        note_launch();
    }
    set_smem(tc::k_leg_analysis_tc, tc::LEG_SMEM);
    const int ntile = (tc_np_max(p) + tc::NMAX - 1) / tc::NMAX;
    dim3 grid((unsigned)((ncol + tc::MTILE - 1) / tc::MTILE), (unsigned)ntile, (unsigned)(2 * (p.lmax + 1)));
    tc::k_leg_analysis_tc<<<grid, tc::NTH, tc::LEG_SMEM, st>>>((const __nv_bfloat16 *)p.d_lamtc, p.d_lamtc_off,
                                                              p.lmax, (int)p.nrn, (rlim + tc::KC - 1) / tc::KC, rlim,
                                                              F, ncol, Ecol, A, Adf, accumulate ? 1 : 0, Eout,
                                                              nzr, p.d_lamtc_live, p.d_err);
    note_launch();
}

}  // namespace sfb

namespace sfb {

int tc_synth_nt(int nrn) {
    const int nt16 = (nrn + 15) & ~15;
    return nt16 < tc::NMAX ? nt16 : tc::NMAX;
}
int tc_synth_nt(const Plan &p) { return tc_synth_nt((int)p.nrn); }

// offsets of every block of a synthesis-layout table over nrn "rings"
// (the rings of the plan, or the output rows of the Gram tables)
int64_t tc_synth_table_offsets(const Plan &p, std::vector<int64_t> &off, int64_t nrn) {
    if (nrn <= 0) nrn = p.nrn;
    const int NT = tc_synth_nt((int)nrn);
    const int ntiles = (int)((nrn + NT - 1) / NT);
    off.assign(2 * (p.lmax + 1) + 1, 0);
    int64_t o = 0;
    for (int z = 0; z < 2 * (p.lmax + 1); ++z) {
        const int m = z >> 1, par = z & 1;
        const int nrows = (m + par <= p.lmax) ? (p.lmax - m - par) / 2 + 1 : 0;
        off[z] = o;
        if (nrows > 0) o += 4LL * NT * ((nrows + tc::KC - 1) / tc::KC) * tc::KC * ntiles;
    }
    off[2 * (p.lmax + 1)] = o;
    return o;
}

namespace tc {
// Live chunk ranges of the sliced tables.  A chunk whose slices are all zero
// contributes exactly zero to every product, so the contractions leave it
// out: per (block z, row tile of NMAX rows) the analysis table's ring chunks,
// per (block z, ring tile) the synthesis table's row chunks.  Ranges [x, y]
// (x > y: no live chunk), preset to {INT_MAX, -1}.
__global__ void k_fill_range(int2 *r, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        r[i] = make_int2(0x7fffffff, -1);
}

// grid (z, ring chunk kc); element e of a plane lies at row (core >> 1) * 8 + ((e & 63) >> 3) with
// core = e >> 6 (core-matrix layout, KC = 16 columns per row group)
__global__ void k_live_analysis(const uint16_t *__restrict__ tab, const int64_t *__restrict__ off, int lmax,
                                int nch, int ntile, int2 *__restrict__ live) {
    __shared__ int any[64];
    const int z = blockIdx.x, kc = blockIdx.y;
    const int m = z >> 1, par = z & 1;
    const int nrows = rows_of(m, par, lmax);
    if (nrows == 0 || kc >= nch) return;
    const int NP = pad16(nrows);
    const uint16_t *base = tab + off[z] + (int64_t)kc * 4 * NP * KC;
    if (threadIdx.x < 64) any[threadIdx.x] = 0;
    __syncthreads();
    for (int e = threadIdx.x; e < 4 * NP * KC; e += blockDim.x) {
        if (base[e] & 0x7fff) {
            const int pe = e % (NP * KC);
            const int li = ((pe >> 6) >> 1) * 8 + ((pe & 63) >> 3);
            any[min(li / NMAX, 63)] = 1;
        }
    }
    __syncthreads();
    if (threadIdx.x < ntile && any[threadIdx.x]) {
        atomicMin(&live[(int64_t)z * ntile + threadIdx.x].x, kc);
        atomicMax(&live[(int64_t)z * ntile + threadIdx.x].y, kc);
    }
}

// grid (z, ring tile nt x row chunk kc)
__global__ void k_live_synthesis(const uint16_t *__restrict__ tab, const int64_t *__restrict__ off, int lmax,
                                 int NT, int ntiles, int nkmax, int2 *__restrict__ live) {
    const int z = blockIdx.x, nt = blockIdx.y / nkmax, kc = blockIdx.y % nkmax;
    const int m = z >> 1, par = z & 1;
    const int nrows = rows_of(m, par, lmax);
    const int nK = (nrows + KC - 1) / KC;
    if (nrows == 0 || kc >= nK) return;
    const uint16_t *base = tab + off[z] + ((int64_t)nt * nK + kc) * 4 * NT * KC;
    int any = 0;
    for (int e = threadIdx.x; e < 4 * NT * KC; e += blockDim.x) any |= base[e] & 0x7fff;
    if (__syncthreads_or(any) && threadIdx.x == 0) {
        atomicMin(&live[(int64_t)z * ntiles + nt].x, kc);
        atomicMax(&live[(int64_t)z * ntiles + nt].y, kc);
    }
}

// Ring DFT spectra that no analysis chunk reads: ring pair r and column block u
// (m in [64 u, 64 u + 63]) are dead when, for every block z of those m and
// every row tile, the chunk of r lies outside the tile's live range.
__global__ void k_dft_dead(const int2 *__restrict__ live, int lmax, int nrn, int ntile, int ntn,
                           unsigned char *__restrict__ dead) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x, u = blockIdx.y;
    if (r >= nrn) return;
    const int kc = r / KC;
    bool d = true;
    for (int m = 64 * u; m <= min(lmax, 64 * u + 63) && d; ++m)
        for (int par = 0; par < 2 && d; ++par) {
            const int z = 2 * m + par;
            if (rows_of(m, par, lmax) == 0) continue;
            for (int t = 0; t < ntile; ++t) {
                const int2 lv = live[(int64_t)z * ntile + t];
                if (kc >= lv.x && kc <= lv.y) d = false;
            }
        }
    dead[(int64_t)r * ntn + u] = d ? 1 : 0;
}
}  // namespace tc

int build_live_ranges(Plan &p, cudaStream_t st) {
    const int nz = 2 * (p.lmax + 1);
    const int ntile_a = (tc_np_max(p) + tc::NMAX - 1) / tc::NMAX;
    const int NT = tc_synth_nt(p);
    const int ntiles_s = (int)((p.nrn + NT - 1) / NT);
    const int nkmax = (int)((p.lmax / 2 + 1 + tc::KC - 1) / tc::KC);
    const int64_t na = (int64_t)nz * ntile_a, ns = (int64_t)nz * ntiles_s;
    if (cudaMalloc(&p.d_lamtc_live, (size_t)(na + ns) * sizeof(int2)) != cudaSuccess) {
        cudaGetLastError();
        p.d_lamtc_live = nullptr;
        return fail(SFB_ENOMEM, "device allocation failed (live chunk ranges)");
    }
    p.device_bytes += (na + ns) * (int64_t)sizeof(int2);
    p.d_lamts_live = p.d_lamtc_live + na;
    tc::k_fill_range<<<(unsigned)((na + ns + 255) / 256), 256, 0, st>>>(p.d_lamtc_live, na + ns);
    note_launch();
    tc::k_live_analysis<<<dim3((unsigned)nz, (unsigned)tc_chunks(p)), 256, 0, st>>>(
        (const uint16_t *)p.d_lamtc, p.d_lamtc_off, p.lmax, tc_chunks(p), ntile_a, p.d_lamtc_live);
    note_launch();
    tc::k_live_synthesis<<<dim3((unsigned)nz, (unsigned)(ntiles_s * nkmax)), 256, 0, st>>>(
        (const uint16_t *)p.d_lamts, p.d_lamts_off, p.lmax, NT, ntiles_s, nkmax, p.d_lamts_live);
    note_launch();
    const int ntn = (p.lmax + 1 + 63) / 64;
    if (cudaMalloc(&p.d_dft_dead, (size_t)p.nrn * ntn) != cudaSuccess) {
        cudaGetLastError();
        p.d_dft_dead = nullptr;
        return fail(SFB_ENOMEM, "device allocation failed (ring DFT dead flags)");
    }
    p.device_bytes += p.nrn * ntn;
    tc::k_dft_dead<<<dim3((unsigned)((p.nrn + 127) / 128), (unsigned)ntn), 128, 0, st>>>(
        p.d_lamtc_live, p.lmax, (int)p.nrn, ntile_a, ntn, p.d_dft_dead);
    note_launch();
    return cudaGetLastError() == cudaSuccess ? SFB_OK : fail(SFB_ECUDA, "live chunk ranges failed");
}

void launch_build_lamts(const Plan &p, const int *Es, cudaStream_t st) {
    dim3 grid(64, (unsigned)(2 * (p.lmax + 1)));
    tc::k_build_lamts<<<grid, 256, 0, st>>>(p.d_lam, p.d_lam_off, p.lmax, (int)p.nrn, tc_synth_nt(p), Es,
                                            p.d_lamts_off, (__nv_bfloat16 *)p.d_lamts);
    note_launch();
}

void launch_leg_synthesis_tc(const Plan &p, const float2 *Adf, int64_t ncol, float *G, cudaStream_t st, int rlim,
                             const int *Ein) {
    const int NT = tc_synth_nt(p);
    if (rlim < 0 || rlim > p.nrn) rlim = (int)p.nrn;
    set_smem(tc::k_leg_synthesis_tc, tc::LEG_SMEM);
    // ring tiles covering the first rlim rings (a tile's rings past rlim are computed as well)
    dim3 grid((unsigned)((ncol + tc::MTILE - 1) / tc::MTILE), (unsigned)((rlim + NT - 1) / NT),
              (unsigned)(2 * (p.lmax + 1)));
    tc::k_leg_synthesis_tc<<<grid, tc::NTH, tc::LEG_SMEM, st>>>((const __nv_bfloat16 *)p.d_lamts, p.d_lamts_off,
                                                               p.lmax, (int)p.nrn, NT, Adf, ncol, G, nullptr, nullptr,
                                                               nullptr, nullptr, Ein, nullptr, p.d_lamts_live, p.d_err);
    note_launch();
}

namespace tc {
__global__ void k_df_to_fp64(const float2 *__restrict__ a, int64_t n, double *__restrict__ out) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float2 v = a[i];
        out[i] = (double)v.x + (double)v.y;
    }
}
}  // namespace tc

void launch_df_to_fp64(const float2 *a, int64_t n, double *out, cudaStream_t st) {
    if (n <= 0) return;
    const int64_t blocks = std::min<int64_t>((n + 255) / 256, 152 * 16);
    tc::k_df_to_fp64<<<(unsigned)blocks, 256, 0, st>>>(a, n, out);
    note_launch();
}

void launch_gram_update(const Plan &p, const double *A, const float2 *Adf, const float2 *A0, int64_t ncol,
                        double *Anew, float2 *Adfnew, cudaStream_t st, const int *Ein, int *Eout) {
    const int NT = tc_synth_nt(p.gram_rows);
    set_smem(tc::k_leg_synthesis_tc, tc::LEG_SMEM);
    dim3 grid((unsigned)((ncol + tc::MTILE - 1) / tc::MTILE), (unsigned)((p.gram_rows + NT - 1) / NT),
              (unsigned)(2 * (p.lmax + 1)));
    tc::k_leg_synthesis_tc<<<grid, tc::NTH, tc::LEG_SMEM, st>>>((const __nv_bfloat16 *)p.d_gramts, p.d_gramts_off,
                                                               p.lmax, p.gram_rows, NT, Adf, ncol, nullptr, A, A0,
                                                               Anew, Adfnew, Ein, Eout, nullptr, p.d_err);
    note_launch();
}

// Gram tables of the alias-free rings r >= p.ral, per block z, stored as the
// deviation from the identity:
//   D_z[li][li'] = sum_r lambda_z(li, r) w n_r cfold_r lambda_z(li', r) - delta(li, li'),
// formed with the FP64 synthesis (of unit coefficient vectors) and analysis
// kernels, then sliced into the synthesis layout with the output rows as rings.
namespace tc {
__global__ void k_unit_alm(int lmax, int R, double *E) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t lmsize = (int64_t)(lmax + 1) * (lmax + 2) / 2;
    if (idx >= lmsize * R) return;
    const int64_t lm = idx / R;
    const int c = (int)(idx - lm * R);
    int l = (int)((sqrt(8.0 * (double)lm + 1.0) - 1.0) / 2.0);
    while ((int64_t)(l + 1) * (l + 2) / 2 <= lm) ++l;
    while ((int64_t)l * (l + 1) / 2 > lm) --l;
    const int m = (int)(lm - (int64_t)l * (l + 1) / 2);
    E[idx] = (c == ((l - m) >> 1)) ? 1.0 : 0.0;
}

__global__ void k_gram_weights(const RingGeom *__restrict__ rings, int nrn, int lmax, int ral, double w, int R,
                               double *G) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t total = (int64_t)2 * (lmax + 1) * nrn * R;
    if (idx >= total) return;
    const int r = (int)((idx / R) % nrn);
    const RingGeom g = rings[r];
    G[idx] = r < ral ? 0.0 : G[idx] * (w * (double)g.nph * g.cfold);
}

__global__ void k_gram_gather(int lmax, int R, const double *__restrict__ A, const int64_t *__restrict__ gram_off,
                              double *__restrict__ gram) {
    const int z = blockIdx.y;
    const int m = z >> 1, par = z & 1;
    const int nrows = rows_of(m, par, lmax);
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < nrows * R; idx += gridDim.x * blockDim.x) {
        const int li = idx / R, ro = idx - li * R;             // input row li, output row ro
        double v = 0.0;
        if (ro < nrows) {
            const int l = m + par + 2 * ro;
            v = A[((int64_t)l * (l + 1) / 2 + m) * R + li] - (ro == li ? 1.0 : 0.0);
        }
        gram[gram_off[z] + (int64_t)li * R + ro] = v;
    }
}
}  // namespace tc

int build_gram_tables(Plan &p, cudaStream_t st) {
    const int R = p.gram_rows;
    const int64_t L1 = p.lmax + 1;
    const int64_t nE = p.lmsize * R, nG = 2 * L1 * p.nrn * R;
    std::vector<int64_t> goff(2 * L1 + 1, 0);
    int64_t o = 0;
    for (int z = 0; z < 2 * L1; ++z) {
        const int m = z >> 1, par = z & 1;
        goff[z] = o;
        o += (int64_t)((m + par <= p.lmax) ? (p.lmax - m - par) / 2 + 1 : 0) * R;
    }
    goff[2 * L1] = o;
    double *E = nullptr, *G = nullptr, *A = nullptr, *gram = nullptr;
    int *Ea = nullptr;
    int64_t *d_goff = nullptr;
    const int nEa = (int)(o / R) + 1, nEs = (int)(2 * L1 * R);
    auto cleanup = [&] {
        cudaFree(E);
        cudaFree(G);
        cudaFree(A);
        cudaFree(gram);
        cudaFree(Ea);
        cudaFree(d_goff);
    };
    if (cudaMalloc(&E, nE * sizeof(double)) != cudaSuccess || cudaMalloc(&G, nG * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&A, nE * sizeof(double)) != cudaSuccess || cudaMalloc(&gram, (o + 1) * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&Ea, (size_t)(nEa + nEs) * sizeof(int)) != cudaSuccess ||
        cudaMalloc(&d_goff, goff.size() * sizeof(int64_t)) != cudaSuccess) {
        cudaGetLastError();
        cleanup();
        return fail(SFB_ENOMEM, "device allocation failed (Gram tables)");
    }
    int *Es = Ea + nEa;
    cudaMemcpy(d_goff, goff.data(), goff.size() * sizeof(int64_t), cudaMemcpyHostToDevice);
    const int32_t prec = p.precision;
    p.precision = SFB_FP64;
    tc::k_unit_alm<<<(unsigned)((nE + 255) / 256), 256, 0, st>>>(p.lmax, R, E);
    note_launch();
    launch_leg_synthesis(p, E, R, G, st);
    tc::k_gram_weights<<<(unsigned)((nG + 255) / 256), 256, 0, st>>>(p.d_rings, (int)p.nrn, p.lmax, p.ral,
                                                                     4.0 * M_PI / (double)p.npix, R, G);
    note_launch();
    launch_leg_analysis(p, G, R, A, false, st);
    p.precision = prec;
    tc::k_gram_gather<<<dim3(16, (unsigned)(2 * L1)), 256, 0, st>>>(p.lmax, R, A, d_goff, gram);
    note_launch();
    tc::k_lam_rowexp<<<dim3(8, (unsigned)(2 * L1)), 256, 0, st>>>(gram, d_goff, p.lmax, R, Ea, Es);
    note_launch();
    std::vector<int64_t> soff;
    const int64_t ssz = tc_synth_table_offsets(p, soff, R);
    int rc = SFB_OK;
    if (cudaMalloc(&p.d_gramts, (size_t)(ssz + 1) * 2) != cudaSuccess ||
        cudaMalloc(&p.d_gramts_off, soff.size() * sizeof(int64_t)) != cudaSuccess) {
        cudaGetLastError();
        rc = fail(SFB_ENOMEM, "device allocation failed (Gram tables)");
    } else {
        p.device_bytes += (ssz + 1) * 2 + (int64_t)(soff.size() * sizeof(int64_t));
        cudaMemcpy(p.d_gramts_off, soff.data(), soff.size() * sizeof(int64_t), cudaMemcpyHostToDevice);
        tc::k_build_lamts<<<dim3(64, (unsigned)(2 * L1)), 256, 0, st>>>(gram, d_goff, p.lmax, R, tc_synth_nt(R), Es,
                                                                        p.d_gramts_off,
                                                                        (__nv_bfloat16 *)p.d_gramts);
        note_launch();
    }
    if (cudaStreamSynchronize(st) != cudaSuccess && rc == SFB_OK)
        rc = fail(SFB_ECUDA, std::string("Gram table setup failed: ") + cudaGetErrorString(cudaGetLastError()));
    if (rc == SFB_OK) {
        // the FP64 tables stay for the few-column (FP64) refinement
        p.d_gram64 = gram;
        p.d_gram_off = d_goff;
        p.device_bytes += (o + 1) * 8 + (int64_t)(goff.size() * sizeof(int64_t));
        gram = nullptr;
        d_goff = nullptr;
    }
    cleanup();
    return rc;
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
