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
//               in registers and writes every basis map element exactly once
//               (coalesced over consecutive pixels; empty bins write zeros,
//               so the maps need no clearing).
// Summation order inside a bin follows the int-atomic ranks, so repeated
// calls agree to rounding, not bit for bit.
//
// Mixed precision stores the maps in FP32.  With a reference angular map C,
// each map is written as the fluctuation D_b - mu_b C, with
// mu_b = <D_b, C> / <C, C> estimated in FP64 on every STATS_STRIDE-th group
// of 32 bins; the caller adds mu_b C_lm back in FP64 after the transform.
// C is the weighted galaxy count map of all radial slots, so it carries the
// mean density and the survey boundary exactly as the galaxies sample them
// (a pixelised mask misses the partly covered boundary pixels).  The FP32
// rounding then scales with the fluctuation, not with the mean density that
// the window term later cancels.
#include <algorithm>

#include "sfb_internal.h"

namespace sfb {

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 16;                    // per thread
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

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
// whose pixel the FP32 evaluation cannot settle goes to fb_list and gets its
// key and rank from k_deposit_keys_fallback (FP64), so no warp runs the FP64
// pixel path for one lane.
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
            fb_list[atomicAdd(fb_count, 1)] = (int32_t)(gbase + i);
        }
    }
    key[i] = k;
    xloc[i] = x;
}

// The galaxies the FP32 pixel evaluation left: exact FP64 pixel, then key and
// rank as above (rtp, key, rank indexed globally).
__global__ void k_deposit_keys_fallback(const double *__restrict__ rtp, int64_t nside, int64_t npix, double rmin,
                                        double rmax, double inv_width, int pieces, int32_t *__restrict__ counts,
                                        int32_t *__restrict__ key, int32_t *__restrict__ rank,
                                        const int32_t *__restrict__ fb_list, const int32_t *__restrict__ fb_count) {
    const int n = *fb_count;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int64_t i = fb_list[t];
        const double r = rtp[3 * i], th = rtp[3 * i + 1], ph = rtp[3 * i + 2];
        const int64_t pix = ang2pix_ring_z(nside, cos(th), ph);
        double x;
        const int slot = slot_of(r, rmin, rmax, inv_width, pieces, x);
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

// bin_moments in double-float on the FP32 units (the sampled mean estimate:
// the summation order, set by the atomic ranks, moves it by ~1e-14 only)
template <int MAXDEG>
__device__ __forceinline__ void bin_moments_df(const double2 *__restrict__ sorted, int64_t g0, int64_t g1, int deg,
                                               double (&out)[MAXDEG + 1]) {
    dfl acc[MAXDEG + 1];
#pragma unroll
    for (int k = 0; k <= MAXDEG; ++k) acc[k] = {0.f, 0.f};
    for (int64_t g = g0; g < g1; ++g) {
        const double2 xw = sorted[g];
        const dfl x = df_of(xw.x);
        dfl q0 = df_of(xw.y), q1 = df_mul(q0, x);
        acc[0] = df_add(acc[0], q0);
        if (MAXDEG >= 1) acc[1] = df_add(acc[1], q1);
#pragma unroll
        for (int k = 1; k < MAXDEG; ++k) {
            if (k >= deg) break;
            const dfl c1 = df_of((double)(2 * k + 1) / (k + 1));
            const dfl c2 = df_of(-(double)k / (k + 1));
            const dfl q2 = df_add(df_mul(c1, df_mul(x, q1)), df_mul(c2, q0));
            acc[k + 1] = df_add(acc[k + 1], q2);
            q0 = q1;
            q1 = q2;
        }
    }
#pragma unroll
    for (int k = 0; k <= MAXDEG; ++k) out[k] = (double)acc[k].hi + (double)acc[k].lo;
}

// Mixed precision: moments with the Legendre recurrence, the sums and the
// fluctuation acc - mu_b ref all in double-float (mudf = mu as hi + lo),
// stored as FP32.
template <int MAXDEG>
__global__ void k_deposit_moments_df(const int32_t *__restrict__ offset, const double2 *__restrict__ sorted,
                                     int64_t npix, int pieces, int deg, int64_t nbasis, const double *__restrict__ ref,
                                     const float2 *__restrict__ mudf, float *__restrict__ maps) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nkeys = (int64_t)(pieces + 2) * npix;
    if (idx >= nkeys) return;
    const int slot = (int)(idx / npix);
    const int64_t pix = idx - (int64_t)slot * npix;
    const int64_t g0 = offset[idx];
    const int64_t g1 = offset[idx + 1];
    const dfl rv = df_of(ref ? ref[pix] : 0.0);
    auto fluct = [&](dfl a, int64_t b) -> float {
        if (ref) {
            const float2 m = mudf[b];
            a = df_add(a, df_neg(df_mul({m.x, m.y}, rv)));
        }
        return a.hi + a.lo;
    };
    if (slot >= pieces) {
        dfl s = {0.f, 0.f};
        for (int64_t g = g0; g < g1; ++g) s = df_add(s, df_of(sorted[g].y));
        const int64_t b = nbasis - 2 + (slot - pieces);
        maps[b * npix + pix] = fluct(s, b);
        return;
    }
    dfl acc[MAXDEG + 1];
#pragma unroll
    for (int k = 0; k <= MAXDEG; ++k) acc[k] = {0.f, 0.f};
    for (int64_t g = g0; g < g1; ++g) {
        const double2 xw = sorted[g];
        const dfl x = df_of(xw.x), w = df_of(xw.y);
        dfl p0 = {1.f, 0.f}, p1 = x;
        acc[0] = df_add(acc[0], w);
        if (MAXDEG >= 1) acc[1] = df_add(acc[1], df_mul(w, x));
#pragma unroll
        for (int k = 1; k < MAXDEG; ++k) {
            if (k >= deg) break;
            // (k+1) P_{k+1} = (2k+1) x P_k - k P_{k-1}, the ratios as double-float constants
            const dfl c1 = df_of((double)(2 * k + 1) / (k + 1));
            const dfl c2 = df_of(-(double)k / (k + 1));
            const dfl p2 = df_add(df_mul(c1, df_mul(x, p1)), df_mul(c2, p0));
            acc[k + 1] = df_add(acc[k + 1], df_mul(w, p2));
            p0 = p1;
            p1 = p2;
        }
    }
    const int64_t b0 = (int64_t)slot * (deg + 1);
    float *base = maps + b0 * npix + pix;
#pragma unroll
    for (int k = 0; k <= MAXDEG; ++k)
        if (k <= deg) base[(int64_t)k * npix] = fluct(acc[k], b0 + k);
}

// The same moments with the block's bins handed to its threads in order of
// decreasing galaxy count (a counting sort of the 128 counts in shared
// memory), so the threads of a warp walk bins of nearly equal length instead
// of waiting on the longest bin of 32 neighbours.  The basis values are
// carried as q_k = w P_k(x) through (k+1) q_{k+1} = (2k+1) x q_k - k q_{k-1}.
// Results pass through shared memory and are written with consecutive
// threads on consecutive pixels.  Needs npix >= 128 (a block spans at most
// two slots).
template <int MAXDEG>
__global__ void __launch_bounds__(128) k_deposit_moments_bal(const int32_t *__restrict__ offset,
                                                             const double2 *__restrict__ sorted, int64_t npix,
                                                             int pieces, int deg, int64_t nbasis,
                                                             const double *__restrict__ ref,
                                                             const float2 *__restrict__ mudf,
                                                             float *__restrict__ maps) {
    __shared__ int hist[64];
    __shared__ int perm[128];
    __shared__ float out[(MAXDEG + 1) * 128];
    const int t = threadIdx.x;
    const int64_t nkeys = (int64_t)(pieces + 2) * npix;
    const int64_t B0 = (int64_t)blockIdx.x * 128;
    const int slot0 = (int)(B0 / npix);
    const int64_t bnd = (int64_t)(slot0 + 1) * npix;
    const int64_t bt = B0 + t;
    const int cnt = bt < nkeys ? offset[bt + 1] - offset[bt] : 0;
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
        const dfl rv = df_of(ref ? ref[pix] : 0.0);
        auto fluct = [&](dfl a, int64_t bi) -> float {
            if (ref) {
                const float2 m = mudf[bi];
                a = df_add(a, df_neg(df_mul({m.x, m.y}, rv)));
            }
            return a.hi + a.lo;
        };
        if (slot >= pieces) {
            dfl sw = {0.f, 0.f};
            for (int64_t g = g0; g < g1; ++g) sw = df_add(sw, df_of(sorted[g].y));
            out[q] = fluct(sw, nbasis - 2 + (slot - pieces));
        } else {
            dfl acc[MAXDEG + 1];
#pragma unroll
            for (int k = 0; k <= MAXDEG; ++k) acc[k] = {0.f, 0.f};
            double2 nxt = g0 < g1 ? sorted[g0] : make_double2(0.0, 0.0);
            for (int64_t g = g0; g < g1; ++g) {
                const double2 xw = nxt;
                if (g + 1 < g1) nxt = sorted[g + 1];          // next galaxy's load overlaps this one's basis
                const dfl x = df_of(xw.x);
                dfl q0 = df_of(xw.y), q1 = df_mul(q0, x);
                acc[0] = df_add(acc[0], q0);
                if (MAXDEG >= 1) acc[1] = df_add(acc[1], q1);
#pragma unroll
                for (int k = 1; k < MAXDEG; ++k) {
                    if (k >= deg) break;
                    const dfl c1 = df_of((double)(2 * k + 1) / (k + 1));
                    const dfl c2 = df_of(-(double)k / (k + 1));
                    const dfl q2 = df_add(df_mul(c1, df_mul(x, q1)), df_mul(c2, q0));
                    acc[k + 1] = df_add(acc[k + 1], q2);
                    q0 = q1;
                    q1 = q2;
                }
            }
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
    float *base = maps + (int64_t)slot * (deg + 1) * npix + pix;
    for (int k = 0; k <= deg; ++k) base[(int64_t)k * npix] = out[k * 128 + t];
}

constexpr int STATS_STRIDE = 32;

// Sampled projections onto ref over the bins of every STATS_STRIDE-th group of
// 32 bins (one warp per block): S[b] += <D_b, ref>, Q[slot] += <ref, ref>.
// A slot-uniform warp reduces through shared memory (lane k sums column k);
// a warp that straddles two slots adds per thread.
template <int MAXDEG>
__global__ void __launch_bounds__(32) k_deposit_stats(const int32_t *__restrict__ offset,
                                                      const double2 *__restrict__ sorted, int64_t npix, int pieces,
                                                      int deg, int64_t nbasis, const double *__restrict__ ref,
                                                      double *__restrict__ S, double *__restrict__ Q) {
    __shared__ double red[32][MAXDEG + 3];
    const int lane = threadIdx.x;
    const int64_t idx = (int64_t)blockIdx.x * STATS_STRIDE * 32 + lane;
    const int64_t nkeys = (int64_t)(pieces + 2) * npix;
    const bool valid = idx < nkeys;
    const int slot = valid ? (int)(idx / npix) : -1;
    const int64_t pix = valid ? idx - (int64_t)slot * npix : 0;
    const double rv = valid ? ref[pix] : 0.0;
    double acc[MAXDEG + 1];
    if (valid) {
        bin_moments_df<MAXDEG>(sorted, offset[idx], offset[idx + 1], slot < pieces ? deg : 0, acc);
    } else {
#pragma unroll
        for (int k = 0; k <= MAXDEG; ++k) acc[k] = 0.0;
    }
    const int nk = slot < 0 ? 0 : (slot < pieces ? deg + 1 : 1);
    const unsigned full = 0xffffffffu;
    const int slot0 = __shfl_sync(full, slot, 0);
    if (__all_sync(full, slot == slot0)) {
        if (slot0 < 0) return;
#pragma unroll
        for (int k = 0; k <= MAXDEG; ++k)
            if (k < nk) red[lane][k] = acc[k] * rv;
        red[lane][nk] = rv * rv;
        __syncwarp();
        for (int k = lane; k <= nk; k += 32) {
            double v = 0.0;
            for (int j = 0; j < 32; ++j) v += red[j][k];
            if (k < nk) atomicAdd(S + basis_of(slot0, k, pieces, deg, nbasis), v);
            else atomicAdd(Q + slot0, v);
        }
    } else if (valid) {
#pragma unroll
        for (int k = 0; k <= MAXDEG; ++k)
            if (k < nk) atomicAdd(S + basis_of(slot, k, pieces, deg, nbasis), acc[k] * rv);
        atomicAdd(Q + slot, rv * rv);
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

// Weighted galaxy count per pixel over all radial slots (FP64).
__global__ void k_weight_map(const int32_t *__restrict__ offset, const double2 *__restrict__ sorted, int64_t npix,
                             int nslots, double *__restrict__ C) {
    const int64_t pix = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= npix) return;
    double s = 0.0;
    for (int sl = 0; sl < nslots; ++sl) {
        const int64_t k = (int64_t)sl * npix + pix;
        for (int64_t g = offset[k]; g < offset[k + 1]; ++g) s += sorted[g].y;
    }
    C[pix] = s;
}

template <int MAXDEG>
static void launch_moments(const Plan &p, const int32_t *counts, const double2 *sorted, const double *ref,
                           const double *mu, const float2 *mudf, double *maps, cudaStream_t st) {
    const int64_t nkeys = (int64_t)(p.pieces + 2) * p.npix;
    const unsigned blocks = (unsigned)((nkeys + 127) / 128);
    if (p.precision == SFB_MIXED && MAXDEG <= 31 && p.npix >= 128)
        k_deposit_moments_bal<MAXDEG><<<blocks, 128, 0, st>>>(counts, sorted, p.npix, p.pieces, p.degree, p.nbasis,
                                                              ref, mudf, reinterpret_cast<float *>(maps));
    else if (p.precision == SFB_MIXED)
        k_deposit_moments_df<MAXDEG><<<blocks, 128, 0, st>>>(counts, sorted, p.npix, p.pieces, p.degree, p.nbasis,
                                                             ref, mudf, reinterpret_cast<float *>(maps));
    else
        k_deposit_moments<MAXDEG, double><<<blocks, 128, 0, st>>>(counts, sorted, p.npix, p.pieces, p.degree,
                                                                  p.nbasis, ref, mu, maps);
    note_launch();
}

template <int MAXDEG>
static void launch_stats(const Plan &p, const int32_t *counts, const double2 *sorted, const double *ref, double *S,
                         double *Q, cudaStream_t st) {
    const int64_t nkeys = (int64_t)(p.pieces + 2) * p.npix;
    const int64_t blocks = (nkeys + 32 * STATS_STRIDE - 1) / (32 * STATS_STRIDE);
    k_deposit_stats<MAXDEG><<<(unsigned)blocks, 32, 0, st>>>(counts, sorted, p.npix, p.pieces, p.degree, p.nbasis,
                                                              ref, S, Q);
    note_launch();
}

int deposit_sorted(Plan &p, const double *rtp, const double *w, int64_t ngal, double *maps, double *ref,
                   double *mu, cudaEvent_t ref_ready, cudaStream_t st, const cudaEvent_t *chunk_ready,
                   int nchunks) {
    const int64_t nkeys = (int64_t)(p.pieces + 2) * p.npix;
    const int64_t nscan = nkeys + 1;            // one extra counter: its exclusive prefix is the total
    const int64_t ntiles = (nscan + SCAN_TILE - 1) / SCAN_TILE;
    // workspace: counters/offsets [nscan] int32, tile sums [ntiles] int32, key and rank [ngal] int32,
    // local coordinate [ngal] double, sorted (x, w) [ngal] double2
    const int64_t ints = nscan + ntiles + 3 * ngal + 1;      // + FP64-pixel list [ngal] and its count
    const int64_t off_x = (ints + 1) / 2;
    int64_t off_sorted = off_x + ngal;
    off_sorted += off_sorted & 1;
    const int64_t off_stats = off_sorted + 2 * ngal + 2;       // S [nbasis], Q [pieces + 2], mudf [nbasis]
    SFB_TRY(grow(p, p.dep, (size_t)(off_stats + 2 * p.nbasis + p.pieces + 2)));
    int32_t *counts = reinterpret_cast<int32_t *>(p.dep.ptr);
    int32_t *tsum = counts + nscan;
    int32_t *key = tsum + ntiles;
    int32_t *rank = key + ngal;
    int32_t *fb_list = rank + ngal;
    int32_t *fb_count = fb_list + ngal;
    double *xloc = p.dep.ptr + off_x;
    double2 *sorted = reinterpret_cast<double2 *>(p.dep.ptr + off_sorted);
    SFB_CUDA_TRY(cudaMemsetAsync(counts, 0, (size_t)nscan * sizeof(int32_t), st));
    SFB_CUDA_TRY(cudaMemsetAsync(fb_count, 0, sizeof(int32_t), st));
    const double inv_width = (double)p.pieces / (p.rmax - p.rmin);
    // keys: in nchunks galaxy ranges, each after its event (the host entry's copy pipeline), or at once
    const int nck = (chunk_ready && nchunks > 0) ? nchunks : 1;
    const int64_t per = (ngal + nck - 1) / nck;
    for (int c = 0; c < nck; ++c) {
        const int64_t g0 = c * per, n = std::min<int64_t>(per, ngal - g0);
        if (chunk_ready && nchunks > 0) SFB_CUDA_TRY(cudaStreamWaitEvent(st, chunk_ready[c], 0));
        if (n <= 0) continue;
        k_deposit_keys<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(rtp + 3 * g0, w ? w + g0 : nullptr, n, g0,
                                                                    p.nside, p.npix, p.rmin, p.rmax, inv_width,
                                                                    p.pieces, counts, key + g0, rank + g0,
                                                                    xloc + g0, fb_list, fb_count, p.d_err);
        note_launch();
    }
    if (ngal > 0) {
        k_deposit_keys_fallback<<<304, 256, 0, st>>>(rtp, p.nside, p.npix, p.rmin, p.rmax, inv_width, p.pieces,
                                                     counts, key, rank, fb_list, fb_count);
        note_launch();
    }
    k_scan_tiles<<<(unsigned)ntiles, SCAN_THREADS, 0, st>>>(counts, nscan, tsum);
    note_launch();
    k_scan_sums<<<1, 1024, 0, st>>>(tsum, ntiles);
    note_launch();
    k_scan_add<<<(unsigned)((nscan + 255) / 256), 256, 0, st>>>(counts, nscan, tsum);
    note_launch();
    if (ngal > 0) {
        k_deposit_scatter<<<(unsigned)((ngal + 255) / 256), 256, 0, st>>>(w, ngal, key, rank, xloc, counts, sorted);
        note_launch();
    }
    if (p.degree > 63) return fail(SFB_ENOTSUP, "radial degree above 63 is not supported by the sorted deposit");
    const bool split = ref != nullptr && p.precision == SFB_MIXED;
    float2 *mudf = reinterpret_cast<float2 *>(p.dep.ptr + off_stats + p.nbasis + p.pieces + 2);
    if (split) {
        k_weight_map<<<(unsigned)((p.npix + 255) / 256), 256, 0, st>>>(counts, sorted, p.npix, p.pieces + 2, ref);
        note_launch();
        if (ref_ready) SFB_CUDA_TRY(cudaEventRecord(ref_ready, st));
        double *S = p.dep.ptr + off_stats;
        double *Q = S + p.nbasis;
        SFB_CUDA_TRY(cudaMemsetAsync(S, 0, (size_t)(p.nbasis + p.pieces + 2) * sizeof(double), st));
        if (p.degree <= 15) launch_stats<15>(p, counts, sorted, ref, S, Q, st);
        else if (p.degree <= 31) launch_stats<31>(p, counts, sorted, ref, S, Q, st);
        else launch_stats<63>(p, counts, sorted, ref, S, Q, st);
        k_mean_finalize<<<(unsigned)((p.nbasis + 127) / 128), 128, 0, st>>>(S, Q, p.pieces, p.degree, p.nbasis, mu,
                                                                           mudf);
        note_launch();
    }
    // moments in FP64 (FP64 path) or double-float (mixed); stored in the transform's precision
    const double *r = split ? ref : nullptr;
    if (p.degree <= 15) launch_moments<15>(p, counts, sorted, r, mu, mudf, maps, st);
    else if (p.degree <= 31) launch_moments<31>(p, counts, sorted, r, mu, mudf, maps, st);
    else launch_moments<63>(p, counts, sorted, r, mu, mudf, maps, st);
    SFB_CUDA_TRY(cudaGetLastError());
    return SFB_OK;
}

}  // namespace sfb
