// Ring Fourier analysis of double-float maps on the tensor cores (mixed
// precision).
//
// For m <= lmax the ring transform is a matrix product: with rows q = (ring,
// map) of one ring class (all rings of equal length n and phase type) and
// pixels j as the K dimension,
//   F_N(q, m) = w sum_j x_N(q, j) e^{-i m (phi0 + 2 pi j / n)},
// and e^{-i m (phi0 + 2 pi j/n)} = T[k] + i T[k + n/2] with
// T[k] = cos(pi k / n), k = m (2 j + t) mod 2n, t = 1 if phi0 = pi/n else 0.
// The product runs on the unweighted table and the epilogue multiplies by the
// quadrature weight w = 4 pi / npix (a double-float constant, one rounding).
// F+ = F_N + F_S and F- = F_N - F_S go to F[parity][m][ring][2 map + re/im],
// the layout of the Legendre stage.
//
// Error-free splitting (the block-floating-point slicing of Ozaki, Ogita,
// Oishi and Rump, "Error-free transformations of matrix multiplication by
// using fast routines of matrix multiplication", Numer. Algorithms 59, 2012):
// every value of a map row is written on the row's common scale 2^E (max|x| <
// 2^E) as x = sum_s a_s 2^(E - 7 - 8 s), s = 0..3, with integers |a_s| <= 128;
// every table value on the table's common scale 2^EB (|T| <= 1 < 2^EB = 2) as
// T = sum_s b_s 2^(EB - 7 - 8 s), |b_0| <= 64, |b_s| <= 128.  Each slice is a
// BF16 value with at most 8 significant bits, and each operand is represented
// to 2^-32 of its scale.  The products of level v = s_a + s_b (v = 0..3; ten
// products) are integers of one unit U 2^(-8 v) per row and go to their own
// FP32 TMEM accumulator; the level-0 sum stays below 2^23 units for rings of
// up to 1024 pixels, so it is exact whatever order or rounding the tensor
// cores use (the level-v sums, v >= 1, carry 2^(-8 v) of the leading one, so
// a rounding there is below 2^-32 of it).  Levels v >= 4 (below 2^-32 of the
// leading products) are dropped.  The epilogue adds the levels and the north/south rows
// with one significant FP32 rounding (TwoSum on the leading level).  The
// table is unweighted so that cos 0 = 1 is exact in one slice: for m = 0
// every pixel shares one table value, and a value far below its ring's
// maximum (a smooth background beside a single galaxy's spike) multiplies
// only the leading slices of it, so a truncated weighted entry would bias the
// m = 0 ring sums coherently.
//
// Tiles: M = 128 rows = 64 (ring, map) pairs x {north, south} (TMEM lanes
// 0-63 north, 64-127 south), N = 128 accumulator columns (64 m values x
// {cos, -sin}), K in chunks of 32 pixels, three shared-memory stages.  By
// default both operands arrive by cp.async.bulk in the core-matrix layout
// the MMAs read: A from the image k_dft_slice_a writes each call (the sliced
// map rows), B from the twiddle image built with the plan.  The variants
// slice A in the producer warps (the map values of the next chunk prefetched
// into registers) or gather B from the ring's sliced table.  TMEM holds the
// four level accumulators (4 x 128 columns).  Every mbarrier wait is bounded; on timeout
// the CTA records ERR_TC_TIMEOUT, waits for its MMAs (bounded again),
// releases TMEM and returns.
//
// Survey footprint: rows that are zero (rings outside the survey, marked by
// the row-exponent pass with ZERO_ROW_E) are never read.  A tile with no live
// row writes zero spectra without MMAs.  Two tiles whose southern rows are all
// zero run as one tile of 128 northern rows (F+ = F- = F_N).  Both are exact.
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>

#include "sfb_internal.h"
#include "tc_common.cuh"

namespace sfb {
namespace dft {

using namespace tc;

constexpr int ZERO_ROW_E = -127;  // row exponent of an all-zero ring row

// w (hi + lo) as a normalised double-float pair: w = (w.x, w.y) a double-float
// constant, the leading product's rounding error kept (TwoProd by FMA)
__device__ __forceinline__ float2 wmul_df(float2 w, float hi, float lo) {
    const float p = w.x * hi;
    const float e = fmaf(w.x, hi, -p);
    const float t = e + fmaf(w.y, hi, w.x * lo);
    const float h = p + t;
    return make_float2(h, t - (h - p));
}
constexpr int KC = 32;            // pixels per chunk
constexpr int NPAIR = 64;         // (ring, map) pairs per CTA
constexpr int NROW = 128;         // A rows (MMA M): pairs x {north, south}
constexpr int NCOL = 128;         // accumulator columns (MMA N)
constexpr int NPROD = 256;        // producers: warps 0-3 build the A rows, warps 4-7 the B rows
constexpr int NTHR = NPROD + 32;  // + the MMA warp (warp 8)
constexpr int NSTAGE = 3;
constexpr uint32_t PLANE = NROW * KC * 2;              // bytes of one sliced plane (A or B)
constexpr uint32_t STAGE = 8 * PLANE;                  // A planes 0..3, B planes 4..7
constexpr size_t SMEM = NSTAGE * (size_t)STAGE + 128;

__device__ __forceinline__ uint32_t core_off(int row, int k) {
    return (uint32_t)((((row >> 3) * (KC / 8) + (k >> 3)) << 7) + ((row & 7) << 4) + ((k & 7) << 1));
}

// slices of 8 double-float values (hi, lo) (see slice_pair_df), packed as 4 words per plane
__device__ __forceinline__ void slice8_df(const float (&h)[8], const float (&l)[8], const float (&C)[4],
                                          uint32_t (&w)[4][4]) {
#pragma unroll
    for (int t = 0; t < 8; t += 2) {
        uint32_t v[4];
        slice_pair_df(h[t], l[t], h[t + 1], l[t + 1], C, v);
#pragma unroll
        for (int s = 0; s < 4; ++s) w[s][t >> 1] = v[s];
    }
}

__device__ __forceinline__ void st_shared_v4(unsigned char *p, const uint32_t (&v)[4]) {
    *reinterpret_cast<uint4 *>(p) = make_uint4(v[0], v[1], v[2], v[3]);
}

// Per (hemisphere, ring, map): E with max |x| < 2^E over the ring, raised by
// ceil(log2 n) - 10 for rings longer than 1024 pixels so that the leading
// products still sum below 2^23 units; ZERO_ROW_E for a row of zeros (a ring
// outside the survey), whose tiles the DFT skips.  A row holding a
// non-finite value keeps an ordinary exponent, so the value reaches the
// spectra and the transform's finiteness check.  erow layout [2][nrn][nmaps];
// nzr[0] / nzr[1] get the first / last ring pair with a non-zero row (preset
// to a large value / -1).  With ring_live, the rows of maps b < nlive on the
// rings marked 0 are zero by construction and are not read.
__global__ void __launch_bounds__(128) k_ring_rowexp(const float2 *__restrict__ maps, int64_t npix, int64_t nmaps,
                                                     const RingGeom *__restrict__ rings, int nrn, int *erow,
                                                     int *nzr, const int *__restrict__ ring_live, int64_t nlive,
                                                     int nrings) {
    const int r = blockIdx.x;
    const int64_t b = (int64_t)blockIdx.y * 4 + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    const RingGeom g = rings[r];
    bool any = false;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        if (b >= nmaps) break;
        if (ring_live && b < nlive && !ring_live[h ? nrings - 1 - r : r]) {
            if (lane == 0) erow[((int64_t)h * nrn + r) * nmaps + b] = ZERO_ROW_E;
            continue;
        }
        const float2 *x = maps + b * npix + (h ? g.start_s : g.start_n);
        float mx = 0.f;
        bool fin = true;
        for (int j = lane; j < g.nph; j += 32) {
            const float2 v = x[j];                       // |hi + lo| < 2^E when |hi| < 2^E
            fin &= isfinite(v.x) && isfinite(v.y);
            mx = fmaxf(mx, fabsf(v.x));
        }
        for (int off = 16; off > 0; off >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
        fin = __all_sync(0xffffffffu, fin);
        int E = scale_exp(mx);
        const int lg = 32 - __clz(g.nph - 1);              // ceil(log2 n)
        E += max(0, lg - 10);
        E = max(-90, min(E, 100));
        if (mx == 0.f && fin) E = ZERO_ROW_E;
        else any = true;
        if (lane == 0) erow[((int64_t)h * nrn + r) * nmaps + b] = E;
    }
    // the ring-pair range: one thread per block, and an atomic only where it moves a bound
    if (__syncthreads_or(any) && threadIdx.x == 0) {
        if (r < *(volatile int *)nzr) atomicMin(nzr, r);
        if (r > *(volatile int *)(nzr + 1)) atomicMax(nzr + 1, r);
    }
}

// A-operand image: the four sliced planes of every live tile and 32-pixel
// chunk, in the shared-memory core-matrix layout the DFT's MMAs read (4 PLANE
// bytes per (class, tile, chunk), at chunk aoff[class] + tile nch + chunk), so
// that the DFT fetches its A operand by bulk copy like its B operand.  The
// rows, exponents and north-only rule are those of k_ring_dft_tc; tiles with
// no live row (the DFT writes their spectra without reading A) are skipped.
// Grid (tiles, classes, groups of SLICE_CPG chunks), one thread per (row,
// 16-pixel half) as the DFT's imaged producers.
constexpr int SLICE_CPG = 4;
__global__ void __launch_bounds__(NPROD) k_dft_slice_a(const float2 *__restrict__ maps, int64_t npix, int64_t nmaps,
                                                        const RingGeom *__restrict__ rings, int nrn,
                                                        const int32_t *__restrict__ cls_rings,
                                                        const int32_t *__restrict__ cls_off,
                                                        const int *__restrict__ erow, const int64_t *__restrict__ aoff,
                                                        unsigned char *__restrict__ aimg) {
    const int cls = blockIdx.y;
    const int rb = cls_off[cls];
    const int64_t npairs = (int64_t)(cls_off[cls + 1] - rb) * nmaps;
    const int ty = blockIdx.x;
    const int64_t pair0 = (int64_t)ty * NPAIR;
    if (pair0 >= npairs || (int)blockIdx.z * SLICE_CPG * KC >= rings[cls_rings[rb]].nph) return;
    const int tid = threadIdx.x;
    bool snz = false;
    if (tid < 2 * NPAIR) {
        const int64_t qq = (int64_t)(ty & ~1) * NPAIR + tid;
        if (qq < npairs) {
            const int rg = cls_rings[rb + (int)(qq / nmaps)];
            if (rings[rg].start_s != rings[rg].start_n)
                snz = erow[((int64_t)nrn + rg) * nmaps + qq % nmaps] != ZERO_ROW_E;
        }
    }
    const bool nonly = !__syncthreads_or(snz);
    if (nonly && (ty & 1)) return;
    const int ti = tid & (NROW - 1), ahalf = (tid >> 7) & 1;
    const int hemi = nonly ? 0 : ti >> 6;
    const int64_t q = pair0 + (nonly ? ti : (ti & (NPAIR - 1)));
    const bool rok = q < npairs;
    int ring = cls_rings[rb];
    int64_t b = 0;
    if (rok) {
        ring = cls_rings[rb + (int)(q / nmaps)];
        b = q % nmaps;
    }
    const RingGeom g = rings[ring];
    const int E = rok ? erow[((int64_t)hemi * nrn + ring) * nmaps + b] : ZERO_ROW_E;
    const bool live = rok && (hemi == 0 || g.start_s != g.start_n) && E != ZERO_ROW_E;
    if (!__syncthreads_or(live)) return;
    const int n = rings[cls_rings[rb]].nph;
    const int nch = (n + KC - 1) / KC;
    const int kc0 = blockIdx.z * SLICE_CPG, kc1 = min(nch, kc0 + SLICE_CPG);
    const float2 *x = maps + b * npix + (hemi ? g.start_s : g.start_n);
    float C[4];
    slice_consts8(E == ZERO_ROW_E ? 0 : E, C);
    unsigned char *dst = aimg + (size_t)(aoff[cls] + (int64_t)ty * nch) * (4 * PLANE);
    for (int kc = kc0; kc < kc1; ++kc) {
        float4 v[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int j = kc * KC + 16 * ahalf + 2 * i;
            v[i] = (live && j < n) ? *reinterpret_cast<const float4 *>(x + j) : make_float4(0.f, 0.f, 0.f, 0.f);
        }
#pragma unroll
        for (int gq = 0; gq < 2; ++gq) {
            const float4 *c4 = v + 4 * gq;
            const float vh[8] = {c4[0].x, c4[0].z, c4[1].x, c4[1].z, c4[2].x, c4[2].z, c4[3].x, c4[3].z};
            const float vl[8] = {c4[0].y, c4[0].w, c4[1].y, c4[1].w, c4[2].y, c4[2].w, c4[3].y, c4[3].w};
            uint32_t w[4][4];
            slice8_df(vh, vl, C, w);
            const uint32_t off = core_off(ti, 16 * ahalf + 8 * gq);
#pragma unroll
            for (int sl = 0; sl < 4; ++sl)
                *reinterpret_cast<uint4 *>(dst + (size_t)kc * (4 * PLANE) + sl * PLANE + off) =
                    make_uint4(w[sl][0], w[sl][1], w[sl][2], w[sl][3]);
        }
    }
}

// IMG: the B operand of every chunk comes from the precomputed image (one
// 32 KB bulk copy per stage, issued by thread 0) and all eight producer warps
// slice the map rows, two threads per row; otherwise warps 4-7 gather B from
// the ring's sliced table.
// AIMG: the A operand comes from the A-operand image by bulk copy (thread 0; with IMG both planes of a
// stage in one transaction, and the producers only release the stages and run the epilogue; without
// IMG warps 4-7 gather the B planes from the ring's table meanwhile).
template <bool IMG, bool AIMG>
__global__ void __launch_bounds__(NTHR, 1) k_ring_dft_tc(const float2 *__restrict__ maps, int64_t npix, int64_t nmaps,
                                                         const RingGeom *__restrict__ rings, int nrn, int lmax,
                                                         const int32_t *__restrict__ cls_rings,
                                                         const int32_t *__restrict__ cls_off,
                                                         const int *__restrict__ erow, const uint2 *__restrict__ dtw,
                                                         const int64_t *__restrict__ dtw_off,
                                                         const unsigned char *__restrict__ img,
                                                         const int64_t *__restrict__ img_off, float2 *__restrict__ F,
                                                         int64_t ldF, float2 wdf, const unsigned char *dead,
                                                         int ntn, const int *span, int rev,
                                                         const int64_t *__restrict__ aoff,
                                                         const unsigned char *__restrict__ aimg, int *err) {
    extern __shared__ __align__(1024) unsigned char smem[];
    // grid (column blocks u, row tiles, classes): the column blocks of one row tile are launched
    // together and read its map rows through L2 once; rev: classes in reverse order (the polar
    // rings, longest first, so that the launch does not end on its longest CTAs)
    const int cls = rev ? (int)(gridDim.z - 1 - blockIdx.z) : (int)blockIdx.z;
    const int rb = cls_off[cls];
    const int64_t npairs = (int64_t)(cls_off[cls + 1] - rb) * nmaps;
    const int ty = blockIdx.y;
    const int64_t pair0 = (int64_t)ty * NPAIR;
    if (pair0 >= npairs) return;
    const int u = blockIdx.x;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // dead: the spectra of ring r and column block u that no analysis chunk reads (lambda is zero in
    // every slice there for all m of the block); a tile pair whose rings are all dead is not computed
    if (dead) {
        bool need = false;
        if (tid < 2 * NPAIR) {
            const int64_t qq = (int64_t)(ty & ~1) * NPAIR + tid;
            if (qq < npairs) need = !dead[(int64_t)cls_rings[rb + (int)(qq / nmaps)] * ntn + u];
        }
        if (!__syncthreads_or(need)) return;
    }
    // north-only tiles: where the south rows of this tile and of its partner tile ty ^ 1 are all zero
    // (southern rings outside the survey), the even tile takes the north rows of both, 128 pairs, with
    // F+ = F- = F_N, and the odd one has nothing left to do
    bool snz = false;
    if (tid < 2 * NPAIR) {
        const int64_t qq = (int64_t)(ty & ~1) * NPAIR + tid;
        if (qq < npairs) {
            const int rg = cls_rings[rb + (int)(qq / nmaps)];
            if (rings[rg].start_s != rings[rg].start_n)
                snz = erow[((int64_t)nrn + rg) * nmaps + qq % nmaps] != ZERO_ROW_E;
        }
    }
    const bool nonly = !__syncthreads_or(snz);
    if (nonly && (ty & 1)) return;
    const int npr = nonly ? 2 * NPAIR : NPAIR;      // (ring, map) pairs of this tile
    const bool prod = tid < NPROD;
    // IMG: all producers build A; else warps 0-3 A, 4-7 B; AIMG: the A planes arrive by bulk copy
    const bool abuild = AIMG ? false : IMG ? prod : tid < NROW;
    const int ti = tid & (NROW - 1);
    const int ahalf = IMG ? (tid >> 7) & 1 : 0;    // IMG: which 16 pixels of the chunk this thread slices
    // barriers: full[s] (8 producer warps + the image copy), empty[s] (MMA commit), done (all MMAs)
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + NSTAGE * STAGE);
    uint64_t *empty = full + NSTAGE;
    uint64_t *done = empty + NSTAGE;
    uint32_t *slot = reinterpret_cast<uint32_t *>(done + 1);
    int *bad = reinterpret_cast<int *>(slot + 1);

    // ring class: all rows share n, the phase type and the table
    const int ring0 = cls_rings[rb];
    const RingGeom g0 = rings[ring0];
    const int n = g0.nph;
    const int ptype = g0.phi0_den != 0 ? 1 : 0;
    const int n2 = 2 * n;
    const uint2 *T = dtw + dtw_off[ring0];
    const int nch = (n + KC - 1) / KC;
    const unsigned char *bimg = IMG ? img + (size_t)(img_off[cls] + (int64_t)u * nch) * (4 * PLANE) : nullptr;
    const unsigned char *atile = AIMG ? aimg + (size_t)(aoff[cls] + (int64_t)ty * nch) * (4 * PLANE) : nullptr;

    // A row ti: pair ti % 64, hemisphere ti / 64 (north-only tiles: pair ti, north)
    const int hemi = nonly ? 0 : ti >> 6;
    const int64_t q = pair0 + (nonly ? ti : (ti & (NPAIR - 1)));
    const bool rok = q < npairs;
    int ring = ring0;
    int64_t b = 0;
    if (rok) {
        ring = cls_rings[rb + (int)(q / nmaps)];
        b = q % nmaps;
    }
    const RingGeom g = rings[ring];
    const int E = rok ? erow[((int64_t)hemi * nrn + ring) * nmaps + b] : ZERO_ROW_E;
    // zero rows are not read (on rings without galaxies they are not even written)
    const bool rowlive = rok && (hemi == 0 || g.start_s != g.start_n) && E != ZERO_ROW_E;
    const bool live = abuild && rowlive;
    const float2 *x = maps + b * npix + (hemi ? g.start_s : g.start_n);
    float C[4];
    slice_consts8(E == ZERO_ROW_E ? 0 : E, C);
    const int L1 = lmax + 1;
    // a tile of zero rows (rings outside the survey) has zero spectra: written without MMAs
    if (!__syncthreads_or(AIMG ? (rowlive && prod) : live)) {
        for (int i = tid; i < 2 * 64 * npr; i += NTHR) {
            const int pr = i % npr, mo = (i / npr) & 63, sg = i / (64 * npr);
            const int mm = 64 * u + mo;
            const int64_t qo = pair0 + pr;
            if (mm > lmax || qo >= npairs) continue;
            const int oring = cls_rings[rb + (int)(qo / nmaps)];
            // unread spectra (outside the span of ring pairs with data, or dead) are not written
            if (span && (oring < span[0] || oring > span[1])) continue;
            if (dead && dead[(int64_t)oring * ntn + u]) continue;
            *reinterpret_cast<float4 *>(F + ((int64_t)(sg * L1 + mm) * nrn + oring) * ldF + 2 * (qo % nmaps)) =
                make_float4(0.f, 0.f, 0.f, 0.f);
        }
        return;
    }

    // B row ti (gather variant): column c = ti -> m = 64 u + c/2, part c&1 (0: cos, 1: -sin)
    const int m = 64 * u + (ti >> 1);
    const bool mok = m <= lmax;
    const int step = (int)((2LL * m) % n2);
    int kidx = (int)(((int64_t)m * ptype + (int64_t)(ti & 1) * (n / 2)) % n2);   // k of pixel j = 0

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                     "r"(512)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int i = 0; i < NSTAGE; ++i) {
            mbar_init(&full[i], NPROD / 32 + ((IMG || AIMG) ? 1 : 0));
            mbar_init(&empty[i], 1);
        }
        mbar_init(done, 1);
        *bad = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *slot;
    const uint32_t id1 = idesc_bf16(NROW, NCOL), id2 = idesc_bf16(NROW, 2 * NCOL);
    int ncopied = 0;                                   // thread 0 (IMG): image chunks whose copy was issued

    if (!prod) {
        // MMA warp: per chunk wait for both operand halves, issue the ten level products of its two K steps
        if (lane == 0) {
            int issued = 0;
            for (int kc = 0; kc < nch; ++kc) {
                const int st = kc % NSTAGE;
                if (*(volatile int *)bad) break;
                if (!mbar_wait(&full[st], (uint32_t)((kc / NSTAGE) & 1))) {
                    atomicExch(bad, 1);
                    break;
                }
                fence_after();
                const uint32_t base = smem_u32(smem + st * STAGE);
                const uint32_t sbo = (KC / 8) * 128;
                // the ten level products as six MMAs (tc_common.cuh); level v at TMEM columns 128 v
#pragma unroll
                for (int ks = 0; ks < KC / 16; ++ks) {
#pragma unroll
                    for (int q = 0; q < NMERGED; ++q) {
                        const bool first = kc == 0 && ks == 0 && mg_first(q);
                        mma_bf16(tmem + (uint32_t)(NCOL * mg_lvl(q)),
                                 smem_desc(base + mg_a(q) * PLANE + ks * 256, 128, sbo),
                                 smem_desc(base + (4 + mg_b(q)) * PLANE + ks * 256, 128, sbo), mg_two(q) ? id2 : id1,
                                 first ? 0u : 1u);
                    }
                }
                mma_commit(&empty[st]);
                ++issued;
            }
            mma_commit(done);
            if (issued != nch) atomicExch(bad, 1);
        }
    } else {
        // double-float map values (hi, lo) of the next PD chunks, two per float4 load (n is a multiple
        // of 4, ring starts are even, so every load is 16-byte aligned)
        constexpr int NV4 = IMG ? 8 : 16;         // float4 loads per thread per chunk (16 or 32 values)
        constexpr int PD = IMG ? 2 : 1;           // chunks loaded ahead
        float4 pre[PD][NV4];
        auto load_chunk = [&](int kc, float4 (&buf)[NV4]) {
#pragma unroll
            for (int i = 0; i < NV4; ++i) {
                const int j = kc * KC + 16 * ahalf + 2 * i;
                buf[i] = (live && j < n) ? *reinterpret_cast<const float4 *>(x + j) : make_float4(0.f, 0.f, 0.f, 0.f);
            }
        };
        auto do_chunk = [&](int kc, float4 (&cur)[NV4]) -> bool {
            const int st = kc % NSTAGE;
            if (kc >= NSTAGE) {
                // the stage is free once the MMAs of chunk kc - NSTAGE completed
                if (*(volatile int *)bad) return false;
                if (!mbar_wait(&empty[st], (uint32_t)(((kc / NSTAGE) - 1) & 1))) {
                    atomicExch(bad, 1);
                    return false;
                }
            }
            unsigned char *sbase = smem + st * STAGE;         // A planes 0..3, B planes 4..7
            const int j0 = kc * KC;
            if (AIMG && tid == 0) {
                // A planes of this chunk (and with IMG the B planes): one bulk copy from each image
                mbar_expect_tx(&full[st], (IMG ? 8 : 4) * PLANE);
                bulk_g2s(sbase, atile + (size_t)kc * (4 * PLANE), 4 * PLANE, &full[st]);
                if (IMG) bulk_g2s(sbase + 4 * PLANE, bimg + (size_t)kc * (4 * PLANE), 4 * PLANE, &full[st]);
                ncopied = kc + 1;
            } else if (IMG && tid == 0) {
                // B planes of this chunk: one bulk copy from the image
                mbar_expect_tx(&full[st], 4 * PLANE);
                bulk_g2s(sbase + 4 * PLANE, bimg + (size_t)kc * (4 * PLANE), 4 * PLANE, &full[st]);
                ncopied = kc + 1;
            }
            if (abuild) {
                // A row: this thread's pixels as groups of 8
#pragma unroll
                for (int gq = 0; gq < NV4 / 4; ++gq) {
                    const float4 *c4 = cur + 4 * gq;
                    const float vh[8] = {c4[0].x, c4[0].z, c4[1].x, c4[1].z, c4[2].x, c4[2].z, c4[3].x, c4[3].z};
                    const float vl[8] = {c4[0].y, c4[0].w, c4[1].y, c4[1].w, c4[2].y, c4[2].w, c4[3].y, c4[3].w};
                    uint32_t w[4][4];
                    slice8_df(vh, vl, C, w);
                    const uint32_t off = core_off(ti, 16 * ahalf + 8 * gq);
#pragma unroll
                    for (int s = 0; s < 4; ++s) st_shared_v4(sbase + s * PLANE + off, w[s]);
                }
                if (kc + PD < nch) load_chunk(kc + PD, cur);
            } else if (!IMG && tid >= NROW) {
                // B row (warps 4-7): table slices at k = m (2 j + t) + part n/2 (mod 2n)
#pragma unroll
                for (int gq = 0; gq < 4; ++gq) {
                    uint32_t w[4][4];
#pragma unroll
                    for (int t = 0; t < 8; t += 2) {
                        const int j = j0 + 8 * gq + t;
                        uint2 e0 = make_uint2(0u, 0u), e1 = make_uint2(0u, 0u);
                        if (mok && j < n) e0 = T[kidx];
                        kidx += step;
                        if (kidx >= n2) kidx -= n2;
                        if (mok && j + 1 < n) e1 = T[kidx];
                        kidx += step;
                        if (kidx >= n2) kidx -= n2;
                        // e.x = slices 0 | 1 << 16, e.y = slices 2 | 3 << 16
                        w[0][t >> 1] = (e0.x & 0xffffu) | (e1.x << 16);
                        w[1][t >> 1] = (e0.x >> 16) | (e1.x & 0xffff0000u);
                        w[2][t >> 1] = (e0.y & 0xffffu) | (e1.y << 16);
                        w[3][t >> 1] = (e0.y >> 16) | (e1.y & 0xffff0000u);
                    }
                    const uint32_t off = core_off(ti, 8 * gq);
#pragma unroll
                    for (int s = 0; s < 4; ++s) st_shared_v4(sbase + (4 + s) * PLANE + off, w[s]);
                }
            }
            fence_proxy_async();
            __syncwarp();
            if (lane == 0) mbar_arrive(&full[st]);      // one arrival per producer warp
            return true;
        };
        if (abuild) {
#pragma unroll
            for (int q = 0; q < PD; ++q)
                if (q < nch) load_chunk(q, pre[q]);
        }
        bool go = true;
        for (int kc = 0; kc < nch && go; kc += PD) {
#pragma unroll
            for (int q = 0; q < PD; ++q)
                if (go && kc + q < nch) go = do_chunk(kc + q, pre[q]);
        }
    }
    // all MMAs complete before TMEM is read or released
    bool ok = mbar_wait(done, 0);
    fence_after();
    ok = __syncthreads_and(ok) && !*(volatile int *)bad;
    if (!ok) {
        if (tid == 0) {
            atomicOr(err, ERR_TC_TIMEOUT);
            // image copies still in flight land before the CTA leaves (bounded waits on their stages)
            for (int kc = ncopied - NSTAGE < 0 ? 0 : ncopied - NSTAGE; kc < ncopied; ++kc)
                mbar_wait(&full[kc % NSTAGE], (uint32_t)((kc / NSTAGE) & 1));
        }
    } else if (prod && nonly) {
        // north-only epilogue: row = pair pair0 + lane index, F+ = F- = lead + rest (the south terms of
        // the general epilogue are zero)
        const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;
        const int half = tid >> 7;
        const int64_t qo = pair0 + (warp & 3) * 32 + lane;
        const bool ook = qo < npairs;
        int oring = ring0;
        int64_t ob = 0;
        if (ook) {
            oring = cls_rings[rb + (int)(qo / nmaps)];
            ob = qo % nmaps;
        }
#pragma unroll 1
        for (int it = 0; it < 4; ++it) {
            const int cg = 4 * half + it;
            float v0[16], v1[16], v2[16], v3[16];
            tmem_ld16(tmem + lane_base + (uint32_t)(16 * cg), v0);
            tmem_ld16(tmem + lane_base + 128u + (uint32_t)(16 * cg), v1);
            tmem_ld16(tmem + lane_base + 256u + (uint32_t)(16 * cg), v2);
            tmem_ld16(tmem + lane_base + 384u + (uint32_t)(16 * cg), v3);
            if (!ook) continue;
#pragma unroll
            for (int t = 0; t < 8; ++t) {
                const int mm = 64 * u + 8 * cg + t;
                if (mm > lmax) break;
                const float2 fr = wmul_df(wdf, v0[2 * t], v1[2 * t] + (v2[2 * t] + v3[2 * t]));
                const float2 fi = wmul_df(wdf, v0[2 * t + 1], v1[2 * t + 1] + (v2[2 * t + 1] + v3[2 * t + 1]));
                const float4 f = make_float4(fr.x, fr.y, fi.x, fi.y);
                *reinterpret_cast<float4 *>(F + ((int64_t)mm * nrn + oring) * ldF + 2 * ob) = f;
                *reinterpret_cast<float4 *>(F + ((int64_t)(L1 + mm) * nrn + oring) * ldF + 2 * ob) = f;
            }
        }
    } else if (prod) {
        // epilogue: per row, lead = level 0 (exact) and rest = level 1 + (level 2 + level 3).  Warps w and
        // w + 4 read the same TMEM lanes (rows) and the column groups cg = it and 4 + it; rows exchange through
        // shared memory; then thread t writes, for column group (t / 128) * 4 + it, F+ (t % 128 < 64) or
        // F- of pair t % 64:  (s, e) = TwoSum(lead_N +- lead_S), F = s + ((rest_N +- rest_S) + e)
        float *xch = reinterpret_cast<float *>(smem);      // [2 halves][16 columns][lead, rest][128 rows]
        const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;
        const int half = tid >> 7;
        const int pr = ti & (NPAIR - 1);
        const int sg = ti >> 6;
        const float sgn = sg ? -1.0f : 1.0f;
        const int64_t qo = pair0 + pr;
        const bool ook = qo < npairs;
        int oring = ring0;
        int64_t ob = 0;
        if (ook) {
            oring = cls_rings[rb + (int)(qo / nmaps)];
            ob = qo % nmaps;
        }
        float *xh = xch + half * (32 * NROW);
#pragma unroll 1
        for (int it = 0; it < 4; ++it) {
            const int cg = 4 * half + it;
            float v0[16], v1[16], v2[16], v3[16];
            tmem_ld16(tmem + lane_base + (uint32_t)(16 * cg), v0);
            tmem_ld16(tmem + lane_base + 128u + (uint32_t)(16 * cg), v1);
            tmem_ld16(tmem + lane_base + 256u + (uint32_t)(16 * cg), v2);
            tmem_ld16(tmem + lane_base + 384u + (uint32_t)(16 * cg), v3);
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                xh[(2 * i) * NROW + ti] = v0[i];
                xh[(2 * i + 1) * NROW + ti] = v1[i] + (v2[i] + v3[i]);
            }
            asm volatile("bar.sync 1, %0;" ::"r"(NPROD) : "memory");     // producer warps only
            if (ook) {
#pragma unroll
                for (int t = 0; t < 8; ++t) {
                    const int mm = 64 * u + 8 * cg + t;
                    if (mm > lmax) break;
                    float2 f[2];
#pragma unroll
                    for (int c2 = 0; c2 < 2; ++c2) {
                        const int i = 2 * t + c2;
                        const float a = xh[(2 * i) * NROW + pr], bb = sgn * xh[(2 * i) * NROW + pr + NPAIR];
                        const float s = a + bb;
                        const float z = s - a;
                        const float e = (a - (s - z)) + (bb - z);
                        f[c2] = wmul_df(wdf, s, (xh[(2 * i + 1) * NROW + pr] + sgn * xh[(2 * i + 1) * NROW + pr + NPAIR]) + e);
                    }
                    *reinterpret_cast<float4 *>(F + ((int64_t)(sg * L1 + mm) * nrn + oring) * ldF + 2 * ob) =
                        make_float4(f[0].x, f[0].y, f[1].x, f[1].y);
                }
            }
            asm volatile("bar.sync 1, %0;" ::"r"(NPROD) : "memory");
        }
    }
    fence_before();
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512) : "memory");
}

// The B operand image: for class c, column block u and chunk kc, the four
// sliced planes of the twiddle tile in the shared-memory core-matrix layout,
// the same bits the gather variant builds (chunk (c, u, kc) at img_off[c] +
// u nch_c + kc, 32 KB each).  Grid (max chunks, classes, column blocks), 128
// threads (one per column).
__global__ void __launch_bounds__(NROW) k_build_dft_image(const RingGeom *__restrict__ rings, int lmax,
                                                          const int32_t *__restrict__ cls_rings,
                                                          const int32_t *__restrict__ cls_off,
                                                          const uint2 *__restrict__ dtw,
                                                          const int64_t *__restrict__ dtw_off,
                                                          const int64_t *__restrict__ img_off,
                                                          unsigned char *__restrict__ img) {
    const int kc = blockIdx.x, cls = blockIdx.y, u = blockIdx.z, ti = threadIdx.x;
    if (img_off[cls] < 0) return;
    const int ring0 = cls_rings[cls_off[cls]];
    const RingGeom g0 = rings[ring0];
    const int n = g0.nph, n2 = 2 * n;
    const int nch = (n + KC - 1) / KC;
    if (kc >= nch) return;
    const int ptype = g0.phi0_den != 0 ? 1 : 0;
    const uint2 *T = dtw + dtw_off[ring0];
    const int m = 64 * u + (ti >> 1);
    const bool mok = m <= lmax;
    unsigned char *dst = img + (size_t)(img_off[cls] + (int64_t)u * nch + kc) * (4 * PLANE);
#pragma unroll 1
    for (int gq = 0; gq < 4; ++gq) {
        uint32_t w[4][4];
        for (int t = 0; t < 8; t += 2) {
            uint2 e[2];
            for (int h = 0; h < 2; ++h) {
                const int j = kc * KC + 8 * gq + t + h;
                const int64_t k = ((int64_t)m * (2 * j + ptype) + (int64_t)(ti & 1) * (n / 2)) % n2;
                e[h] = (mok && j < n) ? T[k] : make_uint2(0u, 0u);
            }
            w[0][t >> 1] = (e[0].x & 0xffffu) | (e[1].x << 16);
            w[1][t >> 1] = (e[0].x >> 16) | (e[1].x & 0xffff0000u);
            w[2][t >> 1] = (e[0].y & 0xffffu) | (e[1].y << 16);
            w[3][t >> 1] = (e[0].y >> 16) | (e[1].y & 0xffff0000u);
        }
        const uint32_t off = core_off(ti, 8 * gq);
        for (int s = 0; s < 4; ++s) st_shared_v4(dst + s * PLANE + off, w[s]);
    }
}

}  // namespace dft

size_t ring_dft_smem() { return dft::SMEM; }

// Image offsets (in 32 KB chunks) per ring class, -1 for a class left to the
// gather variant: the equatorial classes always, the polar ones when
// with_polar.  Returns the total number of chunks; max_nch gets the longest
// class in chunks.
int64_t dft_image_offsets(const Plan &p, const std::vector<int32_t> &crings, const std::vector<int32_t> &coff,
                          bool with_polar, std::vector<int64_t> &off, int &max_nch) {
    const int64_t ntn = (p.lmax + 1 + 63) / 64;
    const int ncls = p.n_polar + p.n_eq_cls;
    off.assign((size_t)ncls, -1);
    int64_t tot = 0;
    max_nch = 1;
    for (int c = 0; c < ncls; ++c) {
        if (c < p.n_polar && !with_polar) continue;
        const int nch = (p.h_rings[crings[coff[c]]].nph + dft::KC - 1) / dft::KC;
        off[c] = tot;
        tot += ntn * nch;
        max_nch = std::max(max_nch, nch);
    }
    return tot;
}

void launch_build_dft_image(const Plan &p, int max_nch, cudaStream_t st) {
    const int ncls = p.n_polar + p.n_eq_cls;
    if (ncls <= 0 || !p.d_dtimg) return;
    dim3 grid((unsigned)max_nch, (unsigned)ncls, (unsigned)((p.lmax + 1 + 63) / 64));
    dft::k_build_dft_image<<<grid, dft::NROW, 0, st>>>(p.d_rings, p.lmax, p.d_cls_rings, p.d_cls_off, p.d_dtw,
                                                       p.d_dtw_off, p.d_dtimg_off, p.d_dtimg);
    note_launch();
}

// Host-side slicing of one table value v (|v| < 2^EB) into four BF16 slices
// b_s 2^(EB - 7 - 8 s), packed as uint2 {s0 | s1 << 16, s2 | s3 << 16}.
static uint16_t bf16_of_exact(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return (uint16_t)(u >> 16);      // f has at most 8 significant bits: truncation is exact
}

uint2 dft_slices(double v, int EB) {
    double y = std::ldexp(v, 7 - EB);
    uint16_t s[4];
    for (int k = 0; k < 4; ++k) {
        const double a = std::nearbyint(y);
        y = (y - a) * 256.0;
        s[k] = bf16_of_exact((float)std::ldexp(a, EB - 7 - 8 * k));
    }
    return make_uint2((uint32_t)s[0] | ((uint32_t)s[1] << 16), (uint32_t)s[2] | ((uint32_t)s[3] << 16));
}

int launch_ring_analysis_tc(Plan &p, const float2 *maps, int64_t nmaps, float2 *F, int *erow, int *nzr,
                            cudaStream_t st, const int *ring_live, int64_t nlive, bool skip_unread) {
    {
        // nzr[0] = 0x7f7f7f7f (above any ring index), nzr[1] = -1
        cudaMemsetAsync(nzr, 0x7f, sizeof(int), st);
        cudaMemsetAsync(nzr + 1, 0xff, sizeof(int), st);
        dim3 grid((unsigned)p.nrn, (unsigned)((nmaps + 3) / 4));
        dft::k_ring_rowexp<<<grid, 128, 0, st>>>(maps, p.npix, nmaps, p.d_rings, (int)p.nrn, erow, nzr, ring_live,
                                                 nlive, (int)(4 * p.nside - 1));
        note_launch();
    }
    set_smem(dft::k_ring_dft_tc<true, true>, dft::SMEM);
    set_smem(dft::k_ring_dft_tc<false, true>, dft::SMEM);
    set_smem(dft::k_ring_dft_tc<true, false>, dft::SMEM);
    set_smem(dft::k_ring_dft_tc<false, false>, dft::SMEM);
    const unsigned ntn = (unsigned)((p.lmax + 1 + 63) / 64);
    const double wq = 4.0 * M_PI / (double)p.npix;
    const float2 wdf = make_float2((float)wq, (float)(wq - (double)(float)wq));
    // skip_unread: the spectra are read only by the first analysis pass, over the span of ring pairs
    // with data and the live chunks, so the others need not be computed or written
    const unsigned char *dead = skip_unread ? p.d_dft_dead : nullptr;
    const int *span = skip_unread ? nzr : nullptr;
    // imaged classes read B from the image, the others gather it from the ring table
    const unsigned mtiles = (unsigned)((nmaps + dft::NPAIR - 1) / dft::NPAIR);
    const int64_t eq_tiles = ((int64_t)p.eq_max_rings * nmaps + dft::NPAIR - 1) / dft::NPAIR;
    // A-operand image for the imaged launches: per-class chunk offsets for this map count, the
    // buffer, and the slicing pass (after the row exponents, on the call's stream)
    // with the A image the polar rings take B from the twiddle image as well (SFBGPU_DFT_POLAR_GATHER:
    // from the L1-resident ring tables, gathered by warps 4-7)
    const bool aimg_polar = p.dft_aimg && p.n_polar > 0 && (p.dft_polar_gather || p.dtimg_polar);
    const bool polar_img = p.dtimg_polar && !(aimg_polar && p.dft_polar_gather);
    const bool aimg_eq = p.dft_aimg && p.d_dtimg != nullptr && p.n_eq_cls > 0;
    // the equatorial classes (equal CTAs, a partly filled last wave) run on the second stream beside
    // the polar rings (longest first), each class group's slicing pass directly before its DFT, so
    // the slicing of one group overlaps the DFT of the other and the tail of each launch the other
    const bool two = p.dft_side && p.n_polar > 0;
    cudaStream_t st_eq = two ? p.dft_side : st;
    if (aimg_polar || aimg_eq) {
        const int ncls = (int)p.h_cls_off.size() - 1;
        if (p.aimg_nmaps != nmaps) {
            p.h_aimg_off.assign(ncls + 1, 0);
            int64_t o = 0;
            for (int c = 0; c < ncls; ++c) {
                p.h_aimg_off[c] = o;
                const int64_t rings_c = p.h_cls_off[c + 1] - p.h_cls_off[c];
                const int64_t tiles = (rings_c * nmaps + dft::NPAIR - 1) / dft::NPAIR;
                const int64_t nph = p.h_rings[p.h_cls_rings[p.h_cls_off[c]]].nph;
                o += tiles * ((nph + dft::KC - 1) / dft::KC);
            }
            p.h_aimg_off[ncls] = o;
            SFB_CUDA_TRY(cudaMemcpyAsync(p.d_aimg_off, p.h_aimg_off.data(), (size_t)(ncls + 1) * sizeof(int64_t),
                                         cudaMemcpyHostToDevice, st));
            p.aimg_nmaps = nmaps;
        }
        SFB_TRY(grow(p, p.aimg, (size_t)(p.h_aimg_off[ncls] * (4 * dft::PLANE) / sizeof(double))));
    }
    if (two) {
        // after the row exponents, the offsets upload and the image's allocation on the call's stream
        cudaEventRecord(p.dft_fork, st);
        cudaStreamWaitEvent(p.dft_side, p.dft_fork, 0);
    }
    if (aimg_polar || aimg_eq) {
        unsigned char *aimg = reinterpret_cast<unsigned char *>(p.aimg.ptr);
        // chunk groups: the longest ring (4 nside pixels) in groups of SLICE_CPG chunks
        const unsigned ngrp = (unsigned)((4 * p.nside + dft::KC * dft::SLICE_CPG - 1) / (dft::KC * dft::SLICE_CPG));
        if (aimg_polar) {
            dft::k_dft_slice_a<<<dim3(mtiles, (unsigned)p.n_polar, ngrp), dft::NPROD, 0, st>>>(
                maps, p.npix, nmaps, p.d_rings, (int)p.nrn, p.d_cls_rings, p.d_cls_off, erow, p.d_aimg_off, aimg);
            note_launch();
        }
        if (aimg_eq) {
            dft::k_dft_slice_a<<<dim3((unsigned)eq_tiles, (unsigned)p.n_eq_cls, ngrp), dft::NPROD, 0, st_eq>>>(
                maps, p.npix, nmaps, p.d_rings, (int)p.nrn, p.d_cls_rings, p.d_cls_off + p.n_polar, erow,
                p.d_aimg_off + p.n_polar, aimg);
            note_launch();
        }
    }
    unsigned char *aimg = reinterpret_cast<unsigned char *>(p.aimg.ptr);
    auto launch = [&](dim3 grid, int c0, bool img, bool ai, int rev, cudaStream_t s) {
        if (!img && ai)
            dft::k_ring_dft_tc<false, true><<<grid, dft::NTHR, dft::SMEM, s>>>(
                maps, p.npix, nmaps, p.d_rings, (int)p.nrn, p.lmax, p.d_cls_rings, p.d_cls_off + c0, erow, p.d_dtw,
                p.d_dtw_off, nullptr, nullptr, F, 2 * nmaps, wdf, dead, (int)ntn, span, rev, p.d_aimg_off + c0, aimg,
                p.d_err);
        else if (img && ai)
            dft::k_ring_dft_tc<true, true><<<grid, dft::NTHR, dft::SMEM, s>>>(
                maps, p.npix, nmaps, p.d_rings, (int)p.nrn, p.lmax, p.d_cls_rings, p.d_cls_off + c0, erow, p.d_dtw,
                p.d_dtw_off, p.d_dtimg, p.d_dtimg_off + c0, F, 2 * nmaps, wdf, dead, (int)ntn, span, rev,
                p.d_aimg_off + c0, aimg, p.d_err);
        else if (img)
            dft::k_ring_dft_tc<true, false><<<grid, dft::NTHR, dft::SMEM, s>>>(
                maps, p.npix, nmaps, p.d_rings, (int)p.nrn, p.lmax, p.d_cls_rings, p.d_cls_off + c0, erow, p.d_dtw,
                p.d_dtw_off, p.d_dtimg, p.d_dtimg_off + c0, F, 2 * nmaps, wdf, dead, (int)ntn, span, rev, nullptr,
                nullptr, p.d_err);
        else
            dft::k_ring_dft_tc<false, false><<<grid, dft::NTHR, dft::SMEM, s>>>(
                maps, p.npix, nmaps, p.d_rings, (int)p.nrn, p.lmax, p.d_cls_rings, p.d_cls_off + c0, erow, p.d_dtw,
                p.d_dtw_off, nullptr, nullptr, F, 2 * nmaps, wdf, dead, (int)ntn, span, rev, nullptr, nullptr,
                p.d_err);
        note_launch();
    };
    launch(dim3(ntn, (unsigned)eq_tiles, (unsigned)p.n_eq_cls), p.n_polar, p.d_dtimg != nullptr, aimg_eq, 0,
           st_eq);
    if (p.n_polar > 0)
        launch(dim3(ntn, mtiles, (unsigned)p.n_polar), 0, polar_img, aimg_polar, 1, st);
    if (two) {
        cudaEventRecord(p.dft_join, p.dft_side);
        cudaStreamWaitEvent(st, p.dft_join, 0);
    }
    return SFB_OK;
}

}  // namespace sfb
