// Galaxy deposit without floating-point atomics.
//
// The deposit D_b[p] = sum_{i in p} w_i phi_b(r_i) is organised as a counting
// sort of the galaxies by key = slot * npix + pixel, where slot is the radial
// piece (0..pieces-1) or one of the two out-of-range slots (r < rmin,
// r > rmax):
//   1. keys:    per galaxy, pixel (bit-exact HEALPix), slot and local
//               coordinate x in [-1, 1]; an int atomic on the key's counter
//               gives the galaxy its rank inside the bin;
//   2. scan:    exclusive prefix sum of the (pieces + 2) * npix counters;
//   3. scatter: (x, w) to its sorted position;
//   4. moments: one thread per (slot, pixel) sums w P_k(x) over its galaxies
//               (mixed precision: in its own shared-memory column) and every
//               basis map element is written exactly once (coalesced over
//               consecutive pixels; empty bins write zeros, so the maps need
//               no clearing).
// Summation order inside a bin follows the int-atomic ranks, so repeated
// calls agree to rounding, not bit for bit.
//
// Mixed precision runs no FP64 instruction per galaxy (integer range tests and
// double-float splits; the records are double-float pairs) and stores the
// maps as double-float pairs (hi, lo), which the ring DFT slices exactly.
// With a reference angular map C, each map is written as the fluctuation
// D_b - mu_b C, with mu_b = <D_b, C> / <C, C> estimated in double-float (sums
// in FP64) on every STATS_STRIDE-th group of 32 bins; the caller adds
// mu_b C_lm back in FP64 after the transform.  Rings holding no galaxy are
// then left unwritten (ring_live), their readers treating them as zero.
// C is the weighted galaxy count map of all radial slots, so it carries the
// mean density and the survey boundary exactly as the galaxies sample them
// (a pixelised mask misses the partly covered boundary pixels).  The reduced
// precision of the transform then scales with the fluctuation, not with the
// mean density that the window term later cancels.
#include <algorithm>
#include <cstring>

#include "sfb_internal.h"

namespace sfb {

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 16;                    // per thread
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

// Double-float arithmetic (value = hi + lo, |lo| <= ulp(hi)/2): ~48
// significant bits from FP32 operations, whose throughput on this GPU is
// many times that of FP64.  TwoSum / TwoProd with FMA (Dekker, Knuth).
struct dfl {
    float hi, lo;
};

__device__ __forceinline__ dfl df_of(double x) {
    const float h = (float)x;
    return {h, (float)(x - (double)h)};
}

__device__ __forceinline__ dfl df_add(dfl a, dfl b) {
    const float s = a.hi + b.hi;
    const float z = s - a.hi;
    const float e = ((a.hi - (s - z)) + (b.hi - z)) + (a.lo + b.lo);
    const float h = s + e;
    return {h, e - (h - s)};
}

__device__ __forceinline__ dfl df_mul(dfl a, dfl b) {
    const float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
    const float h = p + e;
    return {h, e - (h - p)};
}

__device__ __forceinline__ dfl df_neg(dfl a) { return {-a.hi, -a.lo}; }

// The same without the final renormalisation (|lo| may reach a few ulp of
// hi): for chains that renormalise where it matters.
__device__ __forceinline__ dfl dfs_mul(dfl a, dfl b) {
    const float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
    return {p, e};
}

__device__ __forceinline__ dfl dfs_add(dfl a, dfl b) {
    const float s = a.hi + b.hi;
    const float z = s - a.hi;
    return {s, ((a.hi - (s - z)) + (b.hi - z)) + (a.lo + b.lo)};
}

__device__ __forceinline__ dfl df_renorm(dfl a) {
    const float h = a.hi + a.lo;
    return {h, a.lo - (h - a.hi)};
}

// Double -> double-float by integer operations only (no FP64 instruction, whose
// rate on this GPU is a small fraction of the FP32 one): hi = d rounded to the
// nearest FP32 (ties to even, as (float)d), lo = d - hi rounded to FP32, ~48
// significant bits in all.  Finite d; below the FP32 normal range hi is 0
// (sign kept), and lo is 0 for |d| < 2^-75.
__device__ __forceinline__ dfl df_of_bits(double d) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(d);
    const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
    const int e = (int)((b >> 52) & 0x7ff);
    const int fe = e - 1023 + 127;
    if (fe <= 0) return {__uint_as_float(sign), 0.f};
    if (fe >= 255) return {__uint_as_float(sign | 0x7f800000u), 0.f};
    const unsigned long long m = b & 0xfffffffffffffull;
    const unsigned rem = (unsigned)(m & 0x1fffffffu);                 // the 29 bits below FP32
    const unsigned hb = sign | ((unsigned)fe << 23) | (unsigned)(m >> 29);
    const bool up = rem > 0x10000000u || (rem == 0x10000000u && (hb & 1u));
    // a mantissa carry moves into the exponent, as rounding up does
    const float hi = __uint_as_float(hb + (up ? 1u : 0u));
    // d - hi = (rem - up 2^29) 2^(e - 1075); exact scale where 2^(e - 1075) is an FP32 normal
    const int r = (int)rem - (up ? 0x20000000 : 0);
    const int se = e - 1075 + 127;
    float lo = se >= 1 ? (float)r * __uint_as_float((unsigned)se << 23) : 0.f;
    return {hi, sign ? -lo : lo};
}

// IEEE order of finite doubles as signed 64-bit integers (-0 and +0 both 0),
// for range tests without FP64 compares.
__host__ __device__ __forceinline__ long long ord_of(double d) {
    long long b;
    memcpy(&b, &d, 8);
    return b >= 0 ? b : -(b & 0x7fffffffffffffffll);
}

__device__ __forceinline__ bool finite_bits(double d) {
    return (((unsigned long long)__double_as_longlong(d) >> 52) & 0x7ffu) != 0x7ffu;
}

// Slot and local coordinate of radius r: u = (r - rmin) / width in units of
// the pieces (inv_width = pieces / (rmax - rmin), formed once on the host),
// x in [-1, 1] on the piece; slots pieces / pieces + 1 below / above.
__device__ __forceinline__ int slot_of(double r, double rmin, double rmax, double inv_width, int pieces, double &x) {
    x = 0.0;
    if (r < rmin) return pieces;
    if (r > rmax) return pieces + 1;
    const double u = (r - rmin) * inv_width;
    int slot = (int)u;
    if (slot >= pieces) slot = pieces - 1;
    x = 2.0 * (u - (double)slot) - 1.0;
    x = fmin(1.0, fmax(-1.0, x));
    return slot;
}

// Keys of galaxies [0, ngal) of this chunk (global index gbase + i).  A galaxy
// whose pixel the FP32 evaluation cannot settle goes to fb_list with key
// -2 - slot, and gets its key and rank from k_deposit_keys_fallback (FP64
// pixel), so no warp runs the FP64 pixel path for one lane.
__global__ void k_deposit_keys(const double *__restrict__ rtp, const double *__restrict__ wgt, int64_t ngal,
                               int64_t gbase, int64_t nside, int64_t npix, double rmin, double rmax,
                               double inv_width, int pieces, int32_t *__restrict__ counts,
                               int32_t *__restrict__ key, int32_t *__restrict__ rank, double *__restrict__ xloc,
                               int32_t *__restrict__ fb_list, int32_t *__restrict__ fb_count, int *err) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ngal) return;
    const double r = rtp[3 * i], th = rtp[3 * i + 1], ph = rtp[3 * i + 2];
    const double w = wgt ? wgt[i] : 1.0;
    int32_t k = -1;
    double x = 0.0;
    if (!(isfinite(r) && isfinite(th) && isfinite(ph) && isfinite(w))) {
        atomicOr(err, ERR_NONFINITE_INPUT);
    } else if (th < 0.0 || th > M_PI) {
        atomicOr(err, ERR_THETA_RANGE);
    } else {
        const int64_t pix = ang2pix_ring_try(nside, th, ph);
        const int slot = slot_of(r, rmin, rmax, inv_width, pieces, x);
        if (pix >= 0) {
            k = (int32_t)(slot * npix + pix);
            rank[i] = atomicAdd(counts + k, 1);
        } else {
            k = -2 - slot;
            fb_list[atomicAdd(fb_count, 1)] = (int32_t)(gbase + i);
        }
    }
    key[i] = k;
    xloc[i] = x;
}

// Mixed precision keys, with no FP64 instruction: the range tests compare the
// IEEE order of the doubles as integers, theta and phi are rounded to FP32 by
// integer operations for the FP32 pixel evaluation, and the local coordinate
// comes from the double-float split of r (x to ~1e-13, as a float2 pair).
// Slot boundaries follow u = (r - rmin) inv_width in double-float, so a
// galaxy within ~1e-13 of a piece boundary may take the neighbouring piece
// (at x = +-1, where both pieces represent the radial functions).
struct RadialKeyParams {
    long long ord_rmin, ord_rmax;      // ord_of(rmin), ord_of(rmax)
    float rmin_hi, rmin_lo, invw_hi, invw_lo;
};

__global__ void k_deposit_keys_mixed(const double *__restrict__ rtp, const double *__restrict__ wgt, int64_t ngal,
                                     int64_t gbase, int64_t nside, int64_t npix, RadialKeyParams rk, int pieces,
                                     int32_t *__restrict__ counts, int32_t *__restrict__ key,
                                     int32_t *__restrict__ rank, float2 *__restrict__ xdf,
                                     int32_t *__restrict__ fb_list, int32_t *__restrict__ fb_count, int *err) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ngal) return;
    const double r = rtp[3 * i], th = rtp[3 * i + 1], ph = rtp[3 * i + 2];
    const bool wfin = wgt ? finite_bits(wgt[i]) : true;
    constexpr long long ORD_PI = 0x400921fb54442d18ll;          // bits of M_PI
    constexpr long long ORD_4PI = 0x402921fb54442d18ll;         // bits of 4 M_PI
    int32_t k = -1;
    float2 x = make_float2(0.f, 0.f);
    if (!(finite_bits(r) && finite_bits(th) && finite_bits(ph) && wfin)) {
        atomicOr(err, ERR_NONFINITE_INPUT);
    } else {
        const long long oth = ord_of(th);
        if (oth < 0 || oth > ORD_PI) {
            atomicOr(err, ERR_THETA_RANGE);
        } else {
            const long long orr = ord_of(r);
            int slot;
            if (orr < rk.ord_rmin) {
                slot = pieces;
            } else if (orr > rk.ord_rmax) {
                slot = pieces + 1;
            } else {
                const dfl u = df_mul(df_add(df_of_bits(r), {-rk.rmin_hi, -rk.rmin_lo}), {rk.invw_hi, rk.invw_lo});
                float fl = floorf(u.hi);
                if (fl == u.hi && u.lo < 0.f) fl -= 1.f;
                slot = min(max((int)fl, 0), pieces - 1);
                const dfl d = df_add(u, {-(float)slot, 0.f});              // in [0, 1] up to rounding
                dfl xx = df_add({2.f * d.hi, 2.f * d.lo}, {-1.f, 0.f});
                if (xx.hi > 1.f || (xx.hi == 1.f && xx.lo > 0.f)) xx = {1.f, 0.f};
                if (xx.hi < -1.f || (xx.hi == -1.f && xx.lo < 0.f)) xx = {-1.f, 0.f};
                x = make_float2(xx.hi, xx.lo);
            }
            const long long phabs = __double_as_longlong(ph) & 0x7fffffffffffffffll;
            const int64_t pix = (nside <= (int64_t(1) << 16) && phabs <= ORD_4PI)
                                    ? ang2pix_ring_try32(nside, df_of_bits(th).hi, df_of_bits(ph).hi)
                                    : -1;
            if (pix >= 0) {
                k = (int32_t)(slot * npix + pix);
                rank[i] = atomicAdd(counts + k, 1);
            } else {
                k = -2 - slot;
                fb_list[atomicAdd(fb_count, 1)] = (int32_t)(gbase + i);
            }
        }
    }
    key[i] = k;
    xdf[i] = x;
}

// The galaxies the FP32 pixel evaluation left: exact FP64 pixel, then key and
// rank as above with the slot the keys pass found (rtp, key, rank indexed
// globally).
__global__ void k_deposit_keys_fallback(const double *__restrict__ rtp, int64_t nside, int64_t npix,
                                        int32_t *__restrict__ counts, int32_t *__restrict__ key,
                                        int32_t *__restrict__ rank, const int32_t *__restrict__ fb_list,
                                        const int32_t *__restrict__ fb_count) {
    const int n = *fb_count;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int64_t i = fb_list[t];
        const double th = rtp[3 * i + 1], ph = rtp[3 * i + 2];
        const int64_t pix = ang2pix_ring_z(nside, cos(th), ph);
        const int slot = -2 - key[i];
        const int32_t k = (int32_t)(slot * npix + pix);
        rank[i] = atomicAdd(counts + k, 1);
        key[i] = k;
    }
}

// Exclusive scan, tile pass: each block scans SCAN_TILE counters in place and
// writes its total.
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_tiles(int32_t *__restrict__ data, int64_t n,
                                                             int32_t *__restrict__ tile_sums) {
    __shared__ int32_t warp_tot[SCAN_THREADS / 32];
    const int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_ITEMS;
    int32_t v[SCAN_ITEMS];
    int32_t s = 0;
#pragma unroll
    for (int j = 0; j < SCAN_ITEMS; ++j) {
        const int64_t idx = base + j;
        v[j] = idx < n ? data[idx] : 0;
        s += v[j];
    }
    // exclusive scan of thread sums across the block
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int32_t inc = s;
    for (int off = 1; off < 32; off <<= 1) {
        const int32_t t = __shfl_up_sync(0xffffffffu, inc, off);
        if (lane >= off) inc += t;
    }
    if (lane == 31) warp_tot[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        int32_t wv = lane < SCAN_THREADS / 32 ? warp_tot[lane] : 0;
        for (int off = 1; off < 32; off <<= 1) {
            const int32_t t = __shfl_up_sync(0xffffffffu, wv, off);
            if (lane >= off) wv += t;
        }
        if (lane < SCAN_THREADS / 32) warp_tot[lane] = wv;   // inclusive warp prefix
    }
    __syncthreads();
    int32_t run = inc - s + (wid > 0 ? warp_tot[wid - 1] : 0);
#pragma unroll
    for (int j = 0; j < SCAN_ITEMS; ++j) {
        const int64_t idx = base + j;
        if (idx < n) data[idx] = run;
        run += v[j];
    }
    if (threadIdx.x == SCAN_THREADS - 1) tile_sums[blockIdx.x] = run;
}

// Scan of the tile totals by one block (serial over chunks of 1024).
__global__ void k_scan_sums(int32_t *__restrict__ sums, int64_t n) {
    __shared__ int32_t buf[1024];
    __shared__ int32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int64_t c0 = 0; c0 < n; c0 += 1024) {
        const int64_t idx = c0 + threadIdx.x;
        const int32_t v = idx < n ? sums[idx] : 0;
        buf[threadIdx.x] = v;
        __syncthreads();
        for (int off = 1; off < 1024; off <<= 1) {
            const int32_t t = threadIdx.x >= off ? buf[threadIdx.x - off] : 0;
            __syncthreads();
            buf[threadIdx.x] += t;
            __syncthreads();
        }
        const int32_t excl = buf[threadIdx.x] - v + carry;
        if (idx < n) sums[idx] = excl;
        __syncthreads();
        if (threadIdx.x == 1023) carry = excl + v;
        __syncthreads();
    }
}

__global__ void k_scan_add(int32_t *__restrict__ data, int64_t n, const int32_t *__restrict__ tile_sums) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx < n) data[idx] += tile_sums[idx / SCAN_TILE];
}

__global__ void k_deposit_scatter(const double *__restrict__ wgt, int64_t ngal, const int32_t *__restrict__ key,
                                  const int32_t *__restrict__ rank, const double *__restrict__ xloc,
                                  const int32_t *__restrict__ offset, double2 *__restrict__ sorted) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ngal) return;
    const int32_t k = key[i];
    if (k < 0) return;
    const int64_t pos = (int64_t)offset[k] + rank[i];
    sorted[pos] = make_double2(xloc[i], wgt ? wgt[i] : 1.0);
}

// Mixed precision: (x, w) as double-float pairs {x.hi, x.lo, w.hi, w.lo}, w
// split from the double by integer operations.
__global__ void k_deposit_scatter_mixed(const double *__restrict__ wgt, int64_t ngal,
                                        const int32_t *__restrict__ key, const int32_t *__restrict__ rank,
                                        const float2 *__restrict__ xdf, const int32_t *__restrict__ offset,
                                        float4 *__restrict__ sorted) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ngal) return;
    const int32_t k = key[i];
    if (k < 0) return;
    const int64_t pos = (int64_t)offset[k] + rank[i];
    const float2 x = xdf[i];
    const dfl w = wgt ? df_of_bits(wgt[i]) : dfl{1.f, 0.f};
    sorted[pos] = make_float4(x.x, x.y, w.hi, w.lo);
}

// Legendre moments sum_i w_i P_k(x_i), k <= deg, of the galaxies g0..g1-1 of one bin.
template <int MAXDEG>
__device__ __forceinline__ void bin_moments(const double2 *__restrict__ sorted, int64_t g0, int64_t g1, int deg,
                                            double (&acc)[MAXDEG + 1]) {
#pragma unroll
    for (int k = 0; k <= MAXDEG; ++k) acc[k] = 0.0;
    for (int64_t g = g0; g < g1; ++g) {
        const double2 xw = sorted[g];
        const double x = xw.x, w = xw.y;
        double p0 = 1.0, p1 = x;
        acc[0] += w;
        if (MAXDEG >= 1) acc[1] += w * x;
#pragma unroll
        for (int k = 1; k < MAXDEG; ++k) {
            if (k >= deg) break;
            // (k+1) P_{k+1} = (2k+1) x P_k - k P_{k-1}; coefficients fold to constants
            const double p2 = ((double)(2 * k + 1) / (k + 1)) * x * p1 - ((double)k / (k + 1)) * p0;
            acc[k + 1] += w * p2;
            p0 = p1;
            p1 = p2;
        }
    }
}

__device__ __forceinline__ int64_t basis_of(int slot, int k, int pieces, int deg, int64_t nbasis) {
    return slot < pieces ? (int64_t)slot * (deg + 1) + k : nbasis - 2 + (slot - pieces);
}

// One thread per (slot, pixel): Legendre moments of its galaxies, minus
// mu_b ref[pix] when ref is given.
template <int MAXDEG, typename TM>
__global__ void k_deposit_moments(const int32_t *__restrict__ offset, const double2 *__restrict__ sorted,
                                  int64_t npix, int pieces, int deg, int64_t nbasis, const double *__restrict__ ref,
                                  const double *__restrict__ mu, TM *__restrict__ maps) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nkeys = (int64_t)(pieces + 2) * npix;
    if (idx >= nkeys) return;
    const int slot = (int)(idx / npix);
    const int64_t pix = idx - (int64_t)slot * npix;
    const int64_t g0 = offset[idx];
    const int64_t g1 = offset[idx + 1];         // offset[nkeys] = number of keyed galaxies
    const double rv = ref ? ref[pix] : 0.0;
    if (slot >= pieces) {       // constant extrapolation maps (r < rmin, r > rmax)
        double s = 0.0;
        for (int64_t g = g0; g < g1; ++g) s += sorted[g].y;
        const int64_t b = nbasis - 2 + (slot - pieces);
        if (ref) s -= mu[b] * rv;
        maps[b * npix + pix] = (TM)s;
        return;
    }
    double acc[MAXDEG + 1];
    bin_moments<MAXDEG>(sorted, g0, g1, deg, acc);
    const int64_t b0 = (int64_t)slot * (deg + 1);
    TM *base = maps + b0 * npix + pix;
#pragma unroll
    for (int k = 0; k <= MAXDEG; ++k) {
        if (k <= deg) {
            const double v = ref ? acc[k] - mu[b0 + k] * rv : acc[k];
            base[(int64_t)k * npix] = (TM)v;
        }
    }
}


// One step of the basis recurrence on q_k = w P_k(x):
// (k+1) q_{k+1} = (2k+1) x q_k - k q_{k-1}, the ratios as double-float
// constants, every operation unnormalised: where the sum cancels, lo keeps
// its absolute accuracy (~2^-46 of the terms), which is all the moments need
// before their FP32 store.
template <int K>
__device__ __forceinline__ dfl leg_step(dfl x, dfl q1, dfl q0) {
    constexpr double C1 = (double)(2 * K + 1) / (K + 1), C2 = -(double)K / (K + 1);
    constexpr float C1H = (float)C1, C2H = (float)C2;
    constexpr float C1L = (float)(C1 - (double)C1H), C2L = (float)(C2 - (double)C2H);
    return dfs_add(dfs_mul({C1H, C1L}, dfs_mul(x, q1)), dfs_mul({C2H, C2L}, q0));
}

// acc[k+1] += q_{k+1} for K <= k < min(deg, MAXDEG), q0 = q_{K-1}, q1 = q_K
template <int K, int MAXDEG>
__device__ __forceinline__ void leg_chain(dfl x, dfl q0, dfl q1, dfl (&acc)[MAXDEG + 1], int deg) {
    if constexpr (K < MAXDEG) {
        if (K >= deg) return;
        const dfl q2 = leg_step<K>(x, q1, q0);
        acc[K + 1] = dfs_add(acc[K + 1], q2);
        leg_chain<K + 1, MAXDEG>(x, q1, q2, acc, deg);
    }
}

// Moments sum_g w_g P_k(x_g), k <= deg, of one bin in double-float, from the
// pairs of k_deposit_scatter_mixed; the next galaxy's load overlaps this
// one's basis.
template <int MAXDEG>
__device__ __forceinline__ void bin_moments_df(const float4 *__restrict__ sorted, int64_t g0, int64_t g1, int deg,
                                               dfl (&acc)[MAXDEG + 1]) {
#pragma unroll
    for (int k = 0; k <= MAXDEG; ++k) acc[k] = {0.f, 0.f};
    float4 nxt = g0 < g1 ? sorted[g0] : make_float4(0.f, 0.f, 0.f, 0.f);
    for (int64_t g = g0; g < g1; ++g) {
        const float4 v = nxt;
        if (g + 1 < g1) nxt = sorted[g + 1];
        const dfl x = {v.x, v.y};
        dfl q0 = {v.z, v.w}, q1 = dfs_mul(q0, x);
        acc[0] = dfs_add(acc[0], q0);
        if (MAXDEG >= 1) acc[1] = dfs_add(acc[1], q1);
        leg_chain<1, MAXDEG>(x, q0, q1, acc, deg);
    }
#pragma unroll
    for (int k = 0; k <= MAXDEG; ++k) acc[k] = df_renorm(acc[k]);
}

// Mixed precision, one thread per (slot, pixel): the moments and the
// fluctuation acc - mu_b ref all in double-float (mudf = mu and cdf = ref as
// hi + lo pairs), stored as normalised double-float pairs.
template <int MAXDEG>
__global__ void k_deposit_moments_df(const int32_t *__restrict__ offset, const float4 *__restrict__ sorted,
                                     int64_t npix, int pieces, int deg, int64_t nbasis, const float2 *__restrict__ cdf,
                                     const float2 *__restrict__ mudf, float2 *__restrict__ maps) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nkeys = (int64_t)(pieces + 2) * npix;
    if (idx >= nkeys) return;
    const int slot = (int)(idx / npix);
    const int64_t pix = idx - (int64_t)slot * npix;
    const int64_t g0 = offset[idx];
    const int64_t g1 = offset[idx + 1];
    const float2 c = cdf ? cdf[pix] : make_float2(0.f, 0.f);
    const dfl rv = {c.x, c.y};
    auto fluct = [&](dfl a, int64_t b) -> float2 {
        if (cdf) {
            const float2 m = mudf[b];
            a = dfs_add(a, df_neg(dfs_mul({m.x, m.y}, rv)));
        }
        a = df_renorm(a);
        return make_float2(a.hi, a.lo);
    };
    if (slot >= pieces) {
        dfl sw = {0.f, 0.f};
        for (int64_t g = g0; g < g1; ++g) {
            const float4 v = sorted[g];
            sw = df_add(sw, {v.z, v.w});
        }
        const int64_t b = nbasis - 2 + (slot - pieces);
        maps[b * npix + pix] = fluct(sw, b);
        return;
    }
    dfl acc[MAXDEG + 1];
    bin_moments_df<MAXDEG>(sorted, g0, g1, deg, acc);
    const int64_t b0 = (int64_t)slot * (deg + 1);
    float2 *base = maps + b0 * npix + pix;
#pragma unroll
    for (int k = 0; k <= MAXDEG; ++k)
        if (k <= deg) base[(int64_t)k * npix] = fluct(acc[k], b0 + k);
}

// The same moments with the block's bins handed to its threads in order of
// decreasing galaxy count (a counting sort of the 128 counts in shared
// memory), so the threads of a warp walk bins of nearly equal length instead
// of waiting on the longest bin of 32 neighbours.  The basis values are
// carried as q_k = w P_k(x) (leg_step).  Results pass through shared memory
// and are written with consecutive threads on consecutive pixels.  Needs
// npix >= 128 (a block spans at most two slots).
template <int MAXDEG>
__global__ void __launch_bounds__(128) k_deposit_moments_bal(const int32_t *__restrict__ offset,
                                                             const float4 *__restrict__ sorted, int64_t npix,
                                                             int pieces, int deg, int64_t nbasis,
                                                             const float2 *__restrict__ cdf,
                                                             const float2 *__restrict__ mudf,
                                                             float2 *__restrict__ maps, int64_t nside,
                                                             const int *__restrict__ ring_live) {
    __shared__ int hist[64];
    __shared__ int perm[128];
    __shared__ float2 out[(MAXDEG + 1) * 128];
    const int t = threadIdx.x;
    const int64_t nkeys = (int64_t)(pieces + 2) * npix;
    const int64_t B0 = (int64_t)blockIdx.x * 128;
    const int slot0 = (int)(B0 / npix);
    const int64_t bnd = (int64_t)(slot0 + 1) * npix;
    const int64_t bt = B0 + t;
    const int cnt = bt < nkeys ? offset[bt + 1] - offset[bt] : 0;
    // blocks of empty bins on pixels where the reference map is zero (outside the survey) write zeros
    bool busy = cnt != 0;
    if (cdf && bt < nkeys) {
        const int sl = bt < bnd ? slot0 : slot0 + 1;
        busy = busy || cdf[bt - (int64_t)sl * npix].x != 0.f;
    }
    if (!__syncthreads_or(busy)) {
        if (bt >= nkeys) return;
        const int sl = bt < bnd ? slot0 : slot0 + 1;
        const int64_t px = bt - (int64_t)sl * npix;
        // rings without galaxies are not written at all (their readers treat them as zero)
        if (ring_live && !ring_live[ring_of_pixel(nside, px)]) return;
        if (sl >= pieces) {
            maps[(nbasis - 2 + (sl - pieces)) * npix + px] = make_float2(0.f, 0.f);
            return;
        }
        float2 *z = maps + (int64_t)sl * (deg + 1) * npix + px;
        for (int k = 0; k <= deg; ++k) z[(int64_t)k * npix] = make_float2(0.f, 0.f);
        return;
    }
    if (t < 64) hist[t] = 0;
    __syncthreads();
    const int key = 63 - min(cnt, 63);                 // longest bins first
    atomicAdd(&hist[key], 1);
    __syncthreads();
    if (t < 32) {
        const int h0 = hist[2 * t], h1 = hist[2 * t + 1];
        int sc = h0 + h1;
        for (int off = 1; off < 32; off <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, sc, off);
            if (t >= off) sc += v;
        }
        const int base = sc - (h0 + h1);
        hist[2 * t] = base;
        hist[2 * t + 1] = base + h0;
    }
    __syncthreads();
    perm[atomicAdd(&hist[key], 1)] = t;
    __syncthreads();
    const int q = perm[t];
    const int64_t b = B0 + q;
    if (b < nkeys) {
        const int slot = b < bnd ? slot0 : slot0 + 1;
        const int64_t pix = b - (int64_t)slot * npix;
        const int64_t g0 = offset[b], g1 = offset[b + 1];
        const float2 c = cdf ? cdf[pix] : make_float2(0.f, 0.f);
        const dfl rv = {c.x, c.y};
        auto fluct = [&](dfl a, int64_t bi) -> float2 {
            if (cdf) {
                const float2 m = mudf[bi];
                a = dfs_add(a, df_neg(dfs_mul({m.x, m.y}, rv)));
            }
            a = df_renorm(a);
            return make_float2(a.hi, a.lo);
        };
        if (slot >= pieces) {
            dfl sw = {0.f, 0.f};
            for (int64_t g = g0; g < g1; ++g) {
                const float4 v = sorted[g];
                sw = df_add(sw, {v.z, v.w});
            }
            out[q] = fluct(sw, nbasis - 2 + (slot - pieces));
        } else {
            dfl acc[MAXDEG + 1];
            bin_moments_df<MAXDEG>(sorted, g0, g1, deg, acc);
            const int64_t bb = (int64_t)slot * (deg + 1);
#pragma unroll
            for (int k = 0; k <= MAXDEG; ++k)
                if (k <= deg) out[k * 128 + q] = fluct(acc[k], bb + k);
        }
    }
    __syncthreads();
    if (bt >= nkeys) return;
    const int slot = bt < bnd ? slot0 : slot0 + 1;
    const int64_t pix = bt - (int64_t)slot * npix;
    if (slot >= pieces) {
        maps[(nbasis - 2 + (slot - pieces)) * npix + pix] = out[t];
        return;
    }
    float2 *base = maps + (int64_t)slot * (deg + 1) * npix + pix;
    for (int k = 0; k <= deg; ++k) base[(int64_t)k * npix] = out[k * 128 + t];
}

// Shared-memory accumulators for the balanced moments (the default): thread t
// keeps the double-float sums of the bin it walks in column t of acc_s (one
// float2 per degree) instead of 25 register pairs, so a thread needs 48
// registers instead of 117 and twice the warps are resident to cover the
// dependent loads (offsets -> records) and the recurrence's latency.  The
// accesses are explicit shared-memory instructions (volatile asm), so the
// compiler cannot move the sums back into registers.  The arithmetic is that
// of k_deposit_moments_bal operation for operation: for the same order of the
// galaxies within each bin both kernels write the same bits.
__device__ __forceinline__ float2 lds2(uint32_t a) {
    float2 v;
    asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(a));
    return v;
}

__device__ __forceinline__ void sts2(uint32_t a, float2 v) {
    asm volatile("st.shared.v2.f32 [%0], {%1, %2};" ::"r"(a), "f"(v.x), "f"(v.y));
}

// column stride of acc_s between degrees: 128 float2
constexpr uint32_t ACC_DEG_BYTES = 128 * 8;

template <int K, int MAXDEG>
__device__ __forceinline__ void leg_chain_sm(dfl x, dfl q0, dfl q1, uint32_t col, int deg) {
    if constexpr (K < MAXDEG) {
        if (K >= deg) return;
        const uint32_t a = col + (K + 1) * ACC_DEG_BYTES;
        const float2 s = lds2(a);
        const dfl q2 = leg_step<K>(x, q1, q0);
        const dfl r = dfs_add({s.x, s.y}, q2);
        sts2(a, make_float2(r.hi, r.lo));
        leg_chain_sm<K + 1, MAXDEG>(x, q1, q2, col, deg);
    }
}

template <int MAXDEG>
__device__ __forceinline__ void bin_moments_sm(const float4 *__restrict__ sorted, int64_t g0, int64_t g1, int deg,
                                               uint32_t col) {
#pragma unroll
    for (int k = 0; k <= MAXDEG; ++k)
        if (k <= deg) sts2(col + k * ACC_DEG_BYTES, make_float2(0.f, 0.f));
    float4 nxt = g0 < g1 ? sorted[g0] : make_float4(0.f, 0.f, 0.f, 0.f);
    for (int64_t g = g0; g < g1; ++g) {
        const float4 v = nxt;
        if (g + 1 < g1) nxt = sorted[g + 1];
        const dfl x = {v.x, v.y};
        const dfl q0 = {v.z, v.w}, q1 = dfs_mul(q0, x);
        float2 s = lds2(col);
        dfl r = dfs_add({s.x, s.y}, q0);
        sts2(col, make_float2(r.hi, r.lo));
        if (MAXDEG >= 1 && deg >= 1) {
            s = lds2(col + ACC_DEG_BYTES);
            r = dfs_add({s.x, s.y}, q1);
            sts2(col + ACC_DEG_BYTES, make_float2(r.hi, r.lo));
        }
        leg_chain_sm<1, MAXDEG>(x, q0, q1, col, deg);
    }
}

template <int MAXDEG>
__global__ void __launch_bounds__(128, 8) k_deposit_moments_sm(const int32_t *__restrict__ offset,
                                                               const float4 *__restrict__ sorted, int64_t npix,
                                                               int pieces, int deg, int64_t nbasis,
                                                               const float2 *__restrict__ cdf,
                                                               const float2 *__restrict__ mudf,
                                                               float2 *__restrict__ maps, int64_t nside,
                                                               const int *__restrict__ ring_live) {
    __shared__ int hist[64];
    __shared__ int perm[128];
    __shared__ __align__(16) float2 acc_s[(MAXDEG + 1) * 128];
    const int t = threadIdx.x;
    const int64_t nkeys = (int64_t)(pieces + 2) * npix;
    const int64_t B0 = (int64_t)blockIdx.x * 128;
    const int slot0 = (int)(B0 / npix);
    const int64_t bnd = (int64_t)(slot0 + 1) * npix;
    const int64_t bt = B0 + t;
    const int cnt = bt < nkeys ? offset[bt + 1] - offset[bt] : 0;
    bool busy = cnt != 0;
    if (cdf && bt < nkeys) {
        const int sl = bt < bnd ? slot0 : slot0 + 1;
        busy = busy || cdf[bt - (int64_t)sl * npix].x != 0.f;
    }
    if (!__syncthreads_or(busy)) {
        if (bt >= nkeys) return;
        const int sl = bt < bnd ? slot0 : slot0 + 1;
        const int64_t px = bt - (int64_t)sl * npix;
        if (ring_live && !ring_live[ring_of_pixel(nside, px)]) return;
        if (sl >= pieces) {
            maps[(nbasis - 2 + (sl - pieces)) * npix + px] = make_float2(0.f, 0.f);
            return;
        }
        float2 *z = maps + (int64_t)sl * (deg + 1) * npix + px;
        for (int k = 0; k <= deg; ++k) z[(int64_t)k * npix] = make_float2(0.f, 0.f);
        return;
    }
    if (t < 64) hist[t] = 0;
    __syncthreads();
    const int key = 63 - min(cnt, 63);                 // longest bins first
    atomicAdd(&hist[key], 1);
    __syncthreads();
    if (t < 32) {
        const int h0 = hist[2 * t], h1 = hist[2 * t + 1];
        int sc = h0 + h1;
        for (int off = 1; off < 32; off <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, sc, off);
            if (t >= off) sc += v;
        }
        const int base = sc - (h0 + h1);
        hist[2 * t] = base;
        hist[2 * t + 1] = base + h0;
    }
    __syncthreads();
    const int walker = atomicAdd(&hist[key], 1);       // the thread that walks this thread's bin
    perm[walker] = t;
    __syncthreads();
    const uint32_t acc0 = (uint32_t)__cvta_generic_to_shared(acc_s);
    {
        const int64_t b = B0 + perm[t];
        if (b < nkeys) {
            const int slot = b < bnd ? slot0 : slot0 + 1;
            const int64_t g0 = offset[b], g1 = offset[b + 1];
            const uint32_t col = acc0 + t * 8;
            if (slot >= pieces) {
                dfl sw = {0.f, 0.f};
                for (int64_t g = g0; g < g1; ++g) {
                    const float4 v = sorted[g];
                    sw = df_add(sw, {v.z, v.w});
                }
                sts2(col, make_float2(sw.hi, sw.lo));
            } else {
                bin_moments_sm<MAXDEG>(sorted, g0, g1, deg, col);
            }
        }
    }
    __syncthreads();
    if (bt >= nkeys) return;
    // thread t writes its own bin (consecutive threads on consecutive pixels) from the walker's column
    const int slot = bt < bnd ? slot0 : slot0 + 1;
    const int64_t pix = bt - (int64_t)slot * npix;
    const uint32_t src = acc0 + walker * 8;
    const float2 c = cdf ? cdf[pix] : make_float2(0.f, 0.f);
    const dfl rv = {c.x, c.y};
    auto fluct = [&](dfl a, int64_t bi) -> float2 {
        if (cdf) {
            const float2 m = mudf[bi];
            a = dfs_add(a, df_neg(dfs_mul({m.x, m.y}, rv)));
        }
        a = df_renorm(a);
        return make_float2(a.hi, a.lo);
    };
    if (slot >= pieces) {
        const float2 s = lds2(src);
        const int64_t b = nbasis - 2 + (slot - pieces);
        maps[b * npix + pix] = fluct({s.x, s.y}, b);
        return;
    }
    const int64_t bb = (int64_t)slot * (deg + 1);
    float2 *base = maps + bb * npix + pix;
    for (int k = 0; k <= deg; ++k) {
        const float2 s = lds2(src + k * ACC_DEG_BYTES);
        base[(int64_t)k * npix] = fluct(df_renorm({s.x, s.y}), bb + k);
    }
}

constexpr int STATS_STRIDE = 32;

// Sampled projections onto ref over the bins of every STATS_STRIDE-th group of
// 32 bins (one warp per block): S[b] += <D_b, ref>, Q[slot] += <ref, ref>,
// with ref as the double-float pairs cdf.  A slot-uniform warp reduces
// through shared memory in double-float (lane k sums column k) and adds the
// column sums in FP64; a warp that straddles two slots adds per thread.
template <int MAXDEG>
__global__ void __launch_bounds__(32) k_deposit_stats(const int32_t *__restrict__ offset,
                                                      const float4 *__restrict__ sorted, int64_t npix, int pieces,
                                                      int deg, int64_t nbasis, const float2 *__restrict__ cdf,
                                                      double *__restrict__ S, double *__restrict__ Q) {
    __shared__ float2 red[32][MAXDEG + 3];
    const int lane = threadIdx.x;
    const int64_t idx = (int64_t)blockIdx.x * STATS_STRIDE * 32 + lane;
    const int64_t nkeys = (int64_t)(pieces + 2) * npix;
    const bool valid = idx < nkeys;
    const int slot = valid ? (int)(idx / npix) : -1;
    const int64_t pix = valid ? idx - (int64_t)slot * npix : 0;
    const float2 c = valid ? cdf[pix] : make_float2(0.f, 0.f);
    const dfl rv = {c.x, c.y};
    dfl acc[MAXDEG + 1];
    if (valid) {
        bin_moments_df<MAXDEG>(sorted, offset[idx], offset[idx + 1], slot < pieces ? deg : 0, acc);
    } else {
#pragma unroll
        for (int k = 0; k <= MAXDEG; ++k) acc[k] = {0.f, 0.f};
    }
    const int nk = slot < 0 ? 0 : (slot < pieces ? deg + 1 : 1);
    const unsigned full = 0xffffffffu;
    const int slot0 = __shfl_sync(full, slot, 0);
    auto to_d = [](dfl a) { return (double)a.hi + (double)a.lo; };
    if (__all_sync(full, slot == slot0)) {
        if (slot0 < 0) return;
#pragma unroll
        for (int k = 0; k <= MAXDEG; ++k)
            if (k < nk) {
                const dfl v = df_mul(acc[k], rv);
                red[lane][k] = make_float2(v.hi, v.lo);
            }
        const dfl rr = df_mul(rv, rv);
        red[lane][nk] = make_float2(rr.hi, rr.lo);
        __syncwarp();
        for (int k = lane; k <= nk; k += 32) {
            dfl v = {0.f, 0.f};
            for (int j = 0; j < 32; ++j) v = df_add(v, {red[j][k].x, red[j][k].y});
            if (k < nk) atomicAdd(S + basis_of(slot0, k, pieces, deg, nbasis), to_d(v));
            else atomicAdd(Q + slot0, to_d(v));
        }
    } else if (valid) {
#pragma unroll
        for (int k = 0; k <= MAXDEG; ++k)
            if (k < nk) atomicAdd(S + basis_of(slot, k, pieces, deg, nbasis), to_d(df_mul(acc[k], rv)));
        atomicAdd(Q + slot, to_d(df_mul(rv, rv)));
    }
}

// mu[b] = S[b] / Q[slot(b)] (0 where the sampled reference map is zero), and
// the same as a double-float pair in mudf.
__global__ void k_mean_finalize(const double *S, const double *Q, int pieces, int deg, int64_t nbasis, double *mu,
                                float2 *mudf) {
    const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nbasis) return;
    const int64_t npoly = (int64_t)pieces * (deg + 1);
    const int slot = b < npoly ? (int)(b / (deg + 1)) : pieces + (int)(b - npoly);
    const double v = Q[slot] > 0.0 ? S[b] / Q[slot] : 0.0;
    mu[b] = v;
    const float h = (float)v;
    mudf[b] = make_float2(h, (float)(v - (double)h));
}

// Weighted galaxy count per pixel over all radial slots (the reference map of
// the mixed deposit), in double-float from the sorted pairs, stored as the
// FP64 value hi + lo (exact) and as the pair itself.
// ring_live[ring] is set to 1 for every ring holding a galaxy (preset to 0).
__global__ void k_weight_map_mixed(const int32_t *__restrict__ offset, const float4 *__restrict__ sorted,
                                   int64_t nside, int64_t npix, int nslots, double *__restrict__ C,
                                   float2 *__restrict__ cdf, int *__restrict__ ring_live) {
    const int64_t pix = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= npix) return;
    dfl s = {0.f, 0.f};
    bool any = false;
    for (int sl = 0; sl < nslots; ++sl) {
        const int64_t k = (int64_t)sl * npix + pix;
        const int64_t g0 = offset[k], g1 = offset[k + 1];
        any = any || g1 > g0;
        for (int64_t g = g0; g < g1; ++g) {
            const float4 v = sorted[g];
            s = df_add(s, {v.z, v.w});
        }
    }
    C[pix] = (double)s.hi + (double)s.lo;
    cdf[pix] = make_float2(s.hi, s.lo);
    if (any) ring_live[ring_of_pixel(nside, pix)] = 1;
}

// FP64 path: double (x, w); mixed: double-float pairs and the count map as cdf
template <int MAXDEG>
static void launch_moments(const Plan &p, const int32_t *counts, const void *sorted, const double *ref,
                           const double *mu, const float2 *cdf, const float2 *mudf, double *maps, cudaStream_t st,
                           const int *ring_live) {
    const int64_t nkeys = (int64_t)(p.pieces + 2) * p.npix;
    const unsigned blocks = (unsigned)((nkeys + 127) / 128);
    const float4 *s4 = static_cast<const float4 *>(sorted);
    float2 *mf = reinterpret_cast<float2 *>(maps);
    bool done = false;
    if constexpr (MAXDEG <= 31) {
        if (p.precision == SFB_MIXED && p.npix >= 128) {
            if (p.moments_smem)
                k_deposit_moments_sm<MAXDEG><<<blocks, 128, 0, st>>>(counts, s4, p.npix, p.pieces, p.degree,
                                                                     p.nbasis, cdf, mudf, mf, p.nside, ring_live);
            else
                k_deposit_moments_bal<MAXDEG><<<blocks, 128, 0, st>>>(counts, s4, p.npix, p.pieces, p.degree,
                                                                      p.nbasis, cdf, mudf, mf, p.nside, ring_live);
            done = true;
        }
    }
    if (done) {
    } else if (p.precision == SFB_MIXED)
        k_deposit_moments_df<MAXDEG><<<blocks, 128, 0, st>>>(counts, s4, p.npix, p.pieces, p.degree, p.nbasis, cdf,
                                                             mudf, mf);
    else
        k_deposit_moments<MAXDEG, double><<<blocks, 128, 0, st>>>(counts, static_cast<const double2 *>(sorted),
                                                                  p.npix, p.pieces, p.degree, p.nbasis, ref, mu,
                                                                  maps);
    note_launch();
}

template <int MAXDEG>
static void launch_stats(const Plan &p, const int32_t *counts, const float4 *sorted, const float2 *cdf, double *S,
                         double *Q, cudaStream_t st) {
    const int64_t nkeys = (int64_t)(p.pieces + 2) * p.npix;
    const int64_t blocks = (nkeys + 32 * STATS_STRIDE - 1) / (32 * STATS_STRIDE);
    k_deposit_stats<MAXDEG><<<(unsigned)blocks, 32, 0, st>>>(counts, sorted, p.npix, p.pieces, p.degree, p.nbasis,
                                                              cdf, S, Q);
    note_launch();
}

// the moment kernels' degree instances: 15, 24 (the default radial basis), 31, 63
template <typename F>
static void by_degree(int deg, F &&f) {
    if (deg <= 15) f(std::integral_constant<int, 15>());
    else if (deg <= 24) f(std::integral_constant<int, 24>());
    else if (deg <= 31) f(std::integral_constant<int, 31>());
    else f(std::integral_constant<int, 63>());
}

int64_t scan_tile_count(int64_t n) { return (n + SCAN_TILE - 1) / SCAN_TILE; }

void launch_exclusive_scan(int32_t *data, int64_t n, int32_t *tile_sums, cudaStream_t st) {
    const int64_t ntiles = scan_tile_count(n);
    k_scan_tiles<<<(unsigned)ntiles, SCAN_THREADS, 0, st>>>(data, n, tile_sums);
    note_launch();
    k_scan_sums<<<1, 1024, 0, st>>>(tile_sums, ntiles);
    note_launch();
    k_scan_add<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(data, n, tile_sums);
    note_launch();
}

int deposit_sorted(Plan &p, const double *rtp, const double *w, int64_t ngal, double *maps, double *ref,
                   double *mu, cudaEvent_t ref_ready, cudaStream_t st, const cudaEvent_t *chunk_ready,
                   int nchunks, const int **ring_live) {
    const bool mixed = p.precision == SFB_MIXED;
    if (ring_live) *ring_live = nullptr;
    const int64_t nkeys = (int64_t)(p.pieces + 2) * p.npix;
    const int64_t nscan = nkeys + 1;            // one extra counter: its exclusive prefix is the total
    const int64_t ntiles = (nscan + SCAN_TILE - 1) / SCAN_TILE;
    // workspace: counters/offsets [nscan] int32, tile sums [ntiles] int32, key, rank and the FP64-pixel
    // list [ngal] int32 (+ its count), local coordinate [ngal] double (mixed: float2), sorted (x, w) [ngal]
    // double2 (mixed: float4), S [nbasis], Q [pieces + 2], mudf [nbasis] float2, cdf [npix] float2
    const int64_t ints = nscan + ntiles + 3 * ngal + 1;
    const int64_t off_x = (ints + 1) / 2;
    int64_t off_sorted = off_x + ngal;
    off_sorted += off_sorted & 1;
    const int64_t off_stats = off_sorted + 2 * ngal + 2;
    const int64_t off_cdf = off_stats + 2 * p.nbasis + p.pieces + 2;
    const int64_t nrings = 4 * p.nside - 1;
    const int64_t off_live = off_cdf + p.npix;               // ring_live [nrings] int
    SFB_TRY(grow(p, p.dep, (size_t)(off_live + (nrings + 1) / 2)));
    int32_t *counts = reinterpret_cast<int32_t *>(p.dep.ptr);
    int32_t *tsum = counts + nscan;
    int32_t *key = tsum + ntiles;
    int32_t *rank = key + ngal;
    int32_t *fb_list = rank + ngal;
    int32_t *fb_count = fb_list + ngal;
    double *xloc = p.dep.ptr + off_x;
    float2 *xdf = reinterpret_cast<float2 *>(xloc);
    void *sorted = p.dep.ptr + off_sorted;
    float4 *sorted4 = static_cast<float4 *>(sorted);
    float2 *cdf = reinterpret_cast<float2 *>(p.dep.ptr + off_cdf);
    int *live = reinterpret_cast<int *>(p.dep.ptr + off_live);
    SFB_CUDA_TRY(cudaMemsetAsync(counts, 0, (size_t)nscan * sizeof(int32_t), st));
    SFB_CUDA_TRY(cudaMemsetAsync(fb_count, 0, sizeof(int32_t), st));
    const double inv_width = (double)p.pieces / (p.rmax - p.rmin);
    RadialKeyParams rk;
    rk.ord_rmin = ord_of(p.rmin);
    rk.ord_rmax = ord_of(p.rmax);
    rk.rmin_hi = (float)p.rmin;
    rk.rmin_lo = (float)(p.rmin - (double)rk.rmin_hi);
    rk.invw_hi = (float)inv_width;
    rk.invw_lo = (float)(inv_width - (double)rk.invw_hi);
    // keys: in nchunks galaxy ranges, each after its event (the host entry's copy pipeline), or at once
    const int nck = (chunk_ready && nchunks > 0) ? nchunks : 1;
    const int64_t per = (ngal + nck - 1) / nck;
    for (int c = 0; c < nck; ++c) {
        const int64_t g0 = c * per, n = std::min<int64_t>(per, ngal - g0);
        if (chunk_ready && nchunks > 0) SFB_CUDA_TRY(cudaStreamWaitEvent(st, chunk_ready[c], 0));
        if (n <= 0) continue;
        const unsigned nb = (unsigned)((n + 255) / 256);
        if (mixed)
            k_deposit_keys_mixed<<<nb, 256, 0, st>>>(rtp + 3 * g0, w ? w + g0 : nullptr, n, g0, p.nside, p.npix, rk,
                                                     p.pieces, counts, key + g0, rank + g0, xdf + g0, fb_list,
                                                     fb_count, p.d_err);
        else
            k_deposit_keys<<<nb, 256, 0, st>>>(rtp + 3 * g0, w ? w + g0 : nullptr, n, g0, p.nside, p.npix, p.rmin,
                                               p.rmax, inv_width, p.pieces, counts, key + g0, rank + g0, xloc + g0,
                                               fb_list, fb_count, p.d_err);
        note_launch();
    }
    if (ngal > 0) {
        k_deposit_keys_fallback<<<304, 256, 0, st>>>(rtp, p.nside, p.npix, counts, key, rank, fb_list, fb_count);
        note_launch();
    }
    launch_exclusive_scan(counts, nscan, tsum, st);
    if (ngal > 0) {
        if (mixed)
            k_deposit_scatter_mixed<<<(unsigned)((ngal + 255) / 256), 256, 0, st>>>(w, ngal, key, rank, xdf, counts,
                                                                                   sorted4);
        else
            k_deposit_scatter<<<(unsigned)((ngal + 255) / 256), 256, 0, st>>>(w, ngal, key, rank, xloc, counts,
                                                                             static_cast<double2 *>(sorted));
        note_launch();
    }
    if (p.degree > 63) return fail(SFB_ENOTSUP, "radial degree above 63 is not supported by the sorted deposit");
    const bool split = ref != nullptr && mixed;
    float2 *mudf = reinterpret_cast<float2 *>(p.dep.ptr + off_stats + p.nbasis + p.pieces + 2);
    if (split) {
        SFB_CUDA_TRY(cudaMemsetAsync(live, 0, (size_t)nrings * sizeof(int), st));
        k_weight_map_mixed<<<(unsigned)((p.npix + 255) / 256), 256, 0, st>>>(counts, sorted4, p.nside, p.npix,
                                                                            p.pieces + 2, ref, cdf, live);
        note_launch();
        if (ref_ready) SFB_CUDA_TRY(cudaEventRecord(ref_ready, st));
        double *S = p.dep.ptr + off_stats;
        double *Q = S + p.nbasis;
        SFB_CUDA_TRY(cudaMemsetAsync(S, 0, (size_t)(p.nbasis + p.pieces + 2) * sizeof(double), st));
        by_degree(p.degree, [&](auto D) { launch_stats<decltype(D)::value>(p, counts, sorted4, cdf, S, Q, st); });
        k_mean_finalize<<<(unsigned)((p.nbasis + 127) / 128), 128, 0, st>>>(S, Q, p.pieces, p.degree, p.nbasis, mu,
                                                                           mudf);
        note_launch();
    }
    // moments in FP64 (FP64 path) or double-float (mixed); stored in the transform's precision
    const bool skip_empty = split && ring_live && p.npix >= 128 && p.degree <= 31;   // the balanced kernel
    by_degree(p.degree, [&](auto D) {
        launch_moments<decltype(D)::value>(p, counts, sorted, split ? ref : nullptr, mu, split ? cdf : nullptr, mudf,
                                           maps, st, skip_empty ? live : nullptr);
    });
    if (skip_empty) *ring_live = live;
    SFB_CUDA_TRY(cudaGetLastError());
    return SFB_OK;
}

}  // namespace sfb
