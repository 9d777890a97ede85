// Ring Fourier transforms on HEALPix rings (analysis and synthesis direction).
//
// A CTA owns one north ring r and its mirrored south ring (same nph and phi0)
// for a tile of MT maps.  The two real rings are packed as one complex
// sequence z_j = f_N[j] + i f_S[j], so one complex DFT of length n = nph
// yields both spectra.  n = 4i (polar) or 4*nside (equatorial) is factored as
// n = o * 2^s with o odd; the transform is the four-step split
//   X[k1 + o*k2] = sum_{j2} W_P^{j2 k2} W_n^{j2 k1} sum_{j1} W_o^{j1 k1} x[P*j1 + j2]
// (P = 2^s): a direct length-o DFT, a twiddle, then an in-place radix-2 FFT of
// length P in shared memory.  Outputs are the coefficients m = 0..lmax with
// aliasing (bin m mod n) and the ring phase e^{-i m phi0}, which is the exact
// ring sum that libsharp's map2alm performs (reference call site
// src/healpix_helpers.jl:55).
#include "sfb_internal.h"

namespace sfb {

template <typename T>
struct cx {
    T x, y;
};

template <typename T>
__device__ __forceinline__ cx<T> cmul(cx<T> a, cx<T> b) {
    return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}

__device__ __forceinline__ int bitrev(int v, int s) { return s == 0 ? 0 : (int)(__brev((unsigned)v) >> (32 - s)); }

namespace {
// Double-float (FP32 pair) arithmetic for the odd-length stage of the FP64
// transform: FP64 throughput is a small fraction of FP32 on this part, and
// the pair keeps about 48 significant bits.
struct df2 {
    float hi, lo;
};
__device__ __forceinline__ df2 d2_of(double x) {
    const float h = (float)x;
    return {h, (float)(x - (double)h)};
}
__device__ __forceinline__ df2 d2_add(df2 a, df2 b) {
    const float s = a.hi + b.hi;
    const float z = s - a.hi;
    const float e = ((a.hi - (s - z)) + (b.hi - z)) + (a.lo + b.lo);
    const float h = s + e;
    return {h, e - (h - s)};
}
__device__ __forceinline__ df2 d2_mul(df2 a, df2 b) {
    const float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
    const float h = p + e;
    return {h, e - (h - p)};
}
__device__ __forceinline__ df2 d2_neg(df2 a) { return {-a.hi, -a.lo}; }
}  // namespace

// The odd-stage input of the FP64 transform is staged as double-float
// (re.hi, re.lo, im.hi, im.lo); other precisions stage their own type.
template <typename T>
__device__ __forceinline__ void store_src(cx<T> *src, int64_t i, cx<T> v) {
    if constexpr (sizeof(T) == 8) {
        const df2 a = d2_of(v.x), b = d2_of(v.y);
        reinterpret_cast<float4 *>(src)[i] = make_float4(a.hi, a.lo, b.hi, b.lo);
    } else {
        src[i] = v;
    }
}

// Four-step DFT of MT packed sequences held in `src` (natural order, only used
// when o > 1) / `buf`; result in `buf`, element k at (k % o) * P + k / o.
// dir = -1 forward (W = e^{-2 pi i/n}), +1 inverse.  `tw` holds W_n^t.
// FP64 (T = double): the length-o DFTs run in double-float with the odd
// roots W_o^t = W_n^{P t} staged in twd (o entries, double-float); `src` holds
// double-float input (store_src).
template <typename T>
__device__ void four_step(cx<T> *buf, cx<T> *src, const cx<T> *tw, int n, int o, int s, int MT,
                          float4 *twd = nullptr) {
    const int P = n / o;
    if constexpr (sizeof(T) == 8) {
        if (o > 1) {
            for (int t = threadIdx.x; t < o; t += blockDim.x) {
                const cx<T> w = tw[P * t];
                const df2 a = d2_of(w.x), b = d2_of(w.y);
                twd[t] = make_float4(a.hi, a.lo, b.hi, b.lo);
            }
            __syncthreads();
            const float4 *srcd = reinterpret_cast<const float4 *>(src);
            for (int idx = threadIdx.x; idx < MT * n; idx += blockDim.x) {
                const int b = idx / n;
                const int rem = idx - b * n;
                const int k1 = rem / P;
                const int j2 = rem - k1 * P;
                const float4 *x = srcd + (int64_t)b * n;
                df2 ar = {0.f, 0.f}, ai = {0.f, 0.f};
                int e = 0;                    // (j1*k1) mod o, advanced incrementally
                for (int j1 = 0; j1 < o; ++j1) {
                    const float4 v = x[P * j1 + j2];
                    const float4 w = twd[e];
                    const df2 vr = {v.x, v.y}, vi = {v.z, v.w}, wr = {w.x, w.y}, wi = {w.z, w.w};
                    ar = d2_add(ar, d2_add(d2_mul(vr, wr), d2_neg(d2_mul(vi, wi))));
                    ai = d2_add(ai, d2_add(d2_mul(vr, wi), d2_mul(vi, wr)));
                    e += k1;
                    if (e >= o) e -= o;
                }
                cx<T> acc = {(T)((double)ar.hi + (double)ar.lo), (T)((double)ai.hi + (double)ai.lo)};
                acc = cmul(acc, tw[j2 * k1]);   // j2*k1 < n
                buf[(int64_t)b * n + k1 * P + bitrev(j2, s)] = acc;
            }
            __syncthreads();
        }
    } else if (o > 1) {
        for (int idx = threadIdx.x; idx < MT * n; idx += blockDim.x) {
            const int b = idx / n;
            const int rem = idx - b * n;
            const int k1 = rem / P;
            const int j2 = rem - k1 * P;
            const cx<T> *x = src + (int64_t)b * n;
            cx<T> acc = {0, 0};
            int e = 0;                    // (P*j1*k1) mod n, advanced incrementally
            const int step = (int)(((int64_t)P * k1) % n);
            for (int j1 = 0; j1 < o; ++j1) {
                const cx<T> v = x[P * j1 + j2];
                const cx<T> w = tw[e];
                acc.x += v.x * w.x - v.y * w.y;
                acc.y += v.x * w.y + v.y * w.x;
                e += step;
                if (e >= n) e -= n;
            }
            acc = cmul(acc, tw[j2 * k1]);   // j2*k1 < n
            buf[(int64_t)b * n + k1 * P + bitrev(j2, s)] = acc;
        }
        __syncthreads();
    }
    // radix-2 DIT stages over the o sequences of length P in each map
    const int halfP = P >> 1;
    for (int len = 2; len <= P; len <<= 1) {
        const int half = len >> 1;
        const int twstride = n / len;
        for (int idx = threadIdx.x; idx < MT * o * halfP; idx += blockDim.x) {
            const int seq = idx / halfP;      // b * o + k1
            const int u = idx - seq * halfP;
            const int grp = u / half;
            const int pos = u - grp * half;
            const int64_t i0 = (int64_t)seq * P + grp * len + pos;
            const int64_t i1 = i0 + half;
            const cx<T> w = tw[twstride * pos];
            const cx<T> a = buf[i0];
            const cx<T> bb = cmul(buf[i1], w);
            buf[i0] = {a.x + bb.x, a.y + bb.y};
            buf[i1] = {a.x - bb.x, a.y - bb.y};
        }
        __syncthreads();
    }
}

// Twiddles W_n^t = e^{dir 2 pi i t / n} from the plan's FP64 table of
// e^{-2 pi i t / n} (one block of n entries per ring, offset twoff).
template <typename T>
__device__ void fill_twiddles(cx<T> *tw, const double2 *__restrict__ tab, int n, int dir) {
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
        const double2 v = tab[t];
        tw[t] = {(T)v.x, (T)(dir < 0 ? v.y : -v.y)};
    }
}

// maps: FP64 [nmaps][npix]; F: [2][lmax+1][nrn][ldF] real view of complex,
// column 2b / 2b+1 = re / im of map b.
// TI: element type of the input maps; TW: element type of the twiddle / phase
// tables (double2 or float2).  The weighted-phase table holds w e^{-i m phi0}.
template <typename T, typename TI, typename TW>
__global__ void __launch_bounds__(256) k_ring_analysis(const RingGeom *rings, int nrn, int lmax,
                                                       int64_t npix, const TI *maps, int64_t nmaps,
                                                       int MT, T *F, int64_t ldF, int r0,
                                                       const TW *__restrict__ twtab,
                                                       const int64_t *__restrict__ twoff,
                                                       const TW *__restrict__ wphase, int *nzr) {
    extern __shared__ unsigned char smem_raw[];
    const int r = r0 + blockIdx.x;
    const int64_t b0 = (int64_t)blockIdx.y * MT;
    const RingGeom g = rings[r];
    const int n = g.nph;
    const int s = __ffs(n) - 1;
    const int o = n >> s;
    const int P = 1 << s;
    const bool paired = g.start_s != g.start_n;
    cx<T> *tw = reinterpret_cast<cx<T> *>(smem_raw);
    cx<T> *buf = tw + n;
    cx<T> *src = buf + (int64_t)MT * n;
    float4 *twd = reinterpret_cast<float4 *>(src + (int64_t)MT * n);     // odd roots (FP64 transform, o > 1)
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
        const TW v = twtab[twoff[r] + t];
        tw[t] = {(T)v.x, (T)v.y};
    }
    // Reduced precision: the ring sums (bin 0) are accumulated exactly enough
    // in double-float (FP32 TwoSum) and replace the FFT's bin 0.
    constexpr bool reduced = sizeof(T) < sizeof(double);
    __shared__ float ring_hi[2 * 8], ring_lo[2 * 8];
    bool nz = false;
    for (int idx = threadIdx.x; idx < MT * n; idx += blockDim.x) {
        const int b = idx / n;
        const int j = idx - b * n;
        const int64_t mb = b0 + b;
        cx<T> v = {0, 0};
        if (mb < nmaps) {
            v.x = (T)maps[mb * npix + g.start_n + j];
            if (paired) v.y = (T)maps[mb * npix + g.start_s + j];
        }
        nz |= (v.x != (T)0) | (v.y != (T)0);           // NaN counts as non-zero
        if (o > 1) store_src(src, (int64_t)b * n + j, v);
        else buf[(int64_t)b * n + bitrev(j, s)] = v;
    }
    const int L1 = lmax + 1;
    if (!__syncthreads_or(nz)) {
        // both rings are zero in every map of the block (outside the survey): zero spectra, no FFT
        for (int idx = threadIdx.x; idx < MT * L1; idx += blockDim.x) {
            const int m = idx / MT;
            const int64_t mb = b0 + (idx - m * MT);
            if (mb >= nmaps) continue;
            T *dp = F + ((int64_t)(0 * L1 + m) * nrn + r) * ldF + 2 * mb;
            T *dq = F + ((int64_t)(1 * L1 + m) * nrn + r) * ldF + 2 * mb;
            dp[0] = dp[1] = dq[0] = dq[1] = (T)0;
        }
        return;
    }
    if (nzr && threadIdx.x == 0) {   // span of the ring pairs with data (the analysis sums over it only)
        atomicMin(nzr, r);
        atomicMax(nzr + 1, r);
    }
    if (reduced) {
        // one warp per (map, ring of the pair): double-float sum of the staged values
        const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
        for (int q = wid; q < 2 * MT; q += blockDim.x >> 5) {
            const int b = q >> 1, side = q & 1;
            float hi = 0.f, lo = 0.f;
            for (int j = lane; j < n; j += 32) {
                const cx<T> v = (o > 1) ? src[(int64_t)b * n + j] : buf[(int64_t)b * n + bitrev(j, s)];
                const float x = (float)(side ? v.y : v.x);
                const float t = hi + x;
                const float bb = t - hi;
                lo += (hi - (t - bb)) + (x - bb);
                hi = t;
            }
            for (int off = 16; off > 0; off >>= 1) {
                const float oh = __shfl_xor_sync(0xffffffffu, hi, off);
                const float ol = __shfl_xor_sync(0xffffffffu, lo, off);
                const float t = hi + oh;
                const float bb = t - hi;
                lo += ol + (hi - (t - bb)) + (oh - bb);
                hi = t;
            }
            if (lane == 0) {
                ring_hi[q] = hi;
                ring_lo[q] = lo;
            }
        }
        __syncthreads();
    }
    four_step<T>(buf, src, tw, n, o, s, MT, twd);
    // unpack, phase, weight; write F+ and F-
    for (int idx = threadIdx.x; idx < MT * L1; idx += blockDim.x) {
        const int m = idx / MT;
        const int b = idx - m * MT;
        const int64_t mb = b0 + b;
        if (mb >= nmaps) continue;
        const int k = m % n;
        const int nk = (n - k) % n;
        const cx<T> Z = buf[(int64_t)b * n + (k % o) * P + k / o];
        const cx<T> Zn = buf[(int64_t)b * n + (nk % o) * P + nk / o];
        T fnx = (Z.x + Zn.x) * (T)0.5, fny = (Z.y - Zn.y) * (T)0.5;
        T fsx = (Z.y + Zn.y) * (T)0.5, fsy = -(Z.x - Zn.x) * (T)0.5;
        if (reduced && k == 0) {   // bin 0 = ring sums (double-float)
            fnx = (T)(ring_hi[2 * b] + ring_lo[2 * b]);
            fsx = (T)(ring_hi[2 * b + 1] + ring_lo[2 * b + 1]);
            fny = fsy = (T)0;
        }
        const TW ph = wphase[(int64_t)r * L1 + m];           // w e^{-i m phi0}
        const T pc = (T)ph.x, ps = (T)ph.y;
        const T px = fnx + fsx, py = fny + fsy;
        const T qx = fnx - fsx, qy = fny - fsy;
        T *dp = F + ((int64_t)(0 * L1 + m) * nrn + r) * ldF + 2 * mb;
        T *dq = F + ((int64_t)(1 * L1 + m) * nrn + r) * ldF + 2 * mb;
        dp[0] = px * pc - py * ps;
        dp[1] = px * ps + py * pc;
        dq[0] = qx * pc - qy * ps;
        dq[1] = qx * ps + qy * pc;
    }
}

// G: [2][lmax+1][nrn][ldG] parity parts of sum_l lambda_lm a_lm.  Writes the
// real ring values of both rings of the pair into maps (FP64 [nmaps][npix]).
template <typename T>
__global__ void __launch_bounds__(256) k_ring_synthesis(const RingGeom *rings, int nrn, int lmax,
                                                        const T *G, int64_t ldG, int64_t nmaps, int MT,
                                                        int64_t npix, double *maps, int r0,
                                                        const double2 *__restrict__ twtab,
                                                        const int64_t *__restrict__ twoff,
                                                        const double2 *__restrict__ phase) {
    extern __shared__ unsigned char smem_raw[];
    const int r = r0 + blockIdx.x;
    const int64_t b0 = (int64_t)blockIdx.y * MT;
    const RingGeom g = rings[r];
    const int n = g.nph;
    const int s = __ffs(n) - 1;
    const int o = n >> s;
    const int P = 1 << s;
    const bool paired = g.start_s != g.start_n;
    cx<T> *tw = reinterpret_cast<cx<T> *>(smem_raw);
    cx<T> *buf = tw + n;
    cx<T> *src = buf + (int64_t)MT * n;
    float4 *twd = reinterpret_cast<float4 *>(src + (int64_t)MT * n);     // odd roots (o > 1)
    fill_twiddles(tw, twtab + twoff[r], n, +1);
    const int L1 = lmax + 1;
    // spectrum of the packed sequence: c_k = CN_k + i CS_k
    for (int idx = threadIdx.x; idx < MT * n; idx += blockDim.x) {
        const int b = idx / n;
        const int k = idx - b * n;
        const int64_t mb = b0 + b;
        double cnx = 0, cny = 0, csx = 0, csy = 0;
        if (mb < nmaps) {
            // m = k + t n
            for (int m = k; m <= lmax; m += n) {
                const T *gp = G + ((int64_t)(0 * L1 + m) * nrn + r) * ldG + 2 * mb;
                const T *gq = G + ((int64_t)(1 * L1 + m) * nrn + r) * ldG + 2 * mb;
                double gnx = (double)gp[0] + (double)gq[0], gny = (double)gp[1] + (double)gq[1];
                double gsx = (double)gp[0] - (double)gq[0], gsy = (double)gp[1] - (double)gq[1];
                if (m == 0) { gny = 0; gsy = 0; }
                const double2 ph = phase[(int64_t)r * L1 + m];     // e^{-i m phi0}
                const double cs = ph.x, sn = -ph.y;                 // e^{+i m phi0}
                cnx += gnx * cs - gny * sn; cny += gnx * sn + gny * cs;
                csx += gsx * cs - gsy * sn; csy += gsx * sn + gsy * cs;
            }
            // m = -k + t n, m >= 1: conj(G_m) e^{-i m phi0}
            const int kk = (n - k) % n;
            for (int m = (kk == 0 ? n : kk); m <= lmax; m += n) {
                const T *gp = G + ((int64_t)(0 * L1 + m) * nrn + r) * ldG + 2 * mb;
                const T *gq = G + ((int64_t)(1 * L1 + m) * nrn + r) * ldG + 2 * mb;
                const double gnx = (double)gp[0] + (double)gq[0], gny = -((double)gp[1] + (double)gq[1]);
                const double gsx = (double)gp[0] - (double)gq[0], gsy = -((double)gp[1] - (double)gq[1]);
                const double2 ph = phase[(int64_t)r * L1 + m];     // e^{-i m phi0}
                const double cs = ph.x, sn = ph.y;
                cnx += gnx * cs - gny * sn; cny += gnx * sn + gny * cs;
                csx += gsx * cs - gsy * sn; csy += gsx * sn + gsy * cs;
            }
        }
        // c = CN + i CS
        const cx<T> v = {(T)(cnx - csy), (T)(cny + csx)};
        if (o > 1) store_src(src, (int64_t)b * n + k, v);
        else buf[(int64_t)b * n + bitrev(k, s)] = v;
    }
    __syncthreads();
    four_step<T>(buf, src, tw, n, o, s, MT, twd);
    for (int idx = threadIdx.x; idx < MT * n; idx += blockDim.x) {
        const int b = idx / n;
        const int j = idx - b * n;
        const int64_t mb = b0 + b;
        if (mb >= nmaps) continue;
        const cx<T> z = buf[(int64_t)b * n + (j % o) * P + j / o];
        maps[mb * npix + g.start_n + j] = (double)z.x;
        if (paired) maps[mb * npix + g.start_s + j] = (double)z.y;
    }
}

// shared memory of one CTA: twiddles, buf (and src) per map, and with src the
// odd roots (n 16-byte entries at most)
static size_t ring_smem(size_t n, size_t elem, bool two_buffers, int mt) {
    return n * elem * (1 + (two_buffers ? 2 : 1) * (size_t)mt) + (two_buffers ? n * 16 : 0);
}

static int ring_mt(size_t n, size_t elem, bool two_buffers) {
    for (int mt = 8; mt >= 1; mt >>= 1)
        if (ring_smem(n, elem, two_buffers, mt) <= 112 * 1024) return mt;   // <= 2 CTAs per SM
    return 1;
}

// Rings [0, nside-1) are polar (nph = 4i, odd factors possible), rings
// [nside-1, 2*nside) equatorial (nph = 4*nside, one buffer when nside is a
// power of two).  Each group is one launch with its own shared-memory size.
template <typename T, typename TI, typename TW>
static void ring_analysis_t(const Plan &p, const TI *maps, int64_t nmaps, T *F, const TW *tw, const TW *wph,
                            cudaStream_t st, int *nzr = nullptr) {
    const int ns = (int)p.nside;
    const bool pow2 = (ns & (ns - 1)) == 0;
    struct Group { int r0, nr; size_t n; bool two; } groups[2] = {
        {0, ns - 1, (size_t)(4 * (ns - 1)), true},
        {ns - 1, ns + 1, (size_t)(4 * ns), !pow2}};
    for (const Group &gr : groups) {
        if (gr.nr <= 0) continue;
        const int MT = ring_mt(gr.n, sizeof(cx<T>), gr.two);
        const size_t smem = ring_smem(gr.n, sizeof(cx<T>), gr.two, MT);
        set_smem(k_ring_analysis<T, TI, TW>, smem);
        dim3 grid((unsigned)gr.nr, (unsigned)((nmaps + MT - 1) / MT));
        k_ring_analysis<T, TI, TW><<<grid, 256, smem, st>>>(p.d_rings, (int)p.nrn, p.lmax, p.npix, maps, nmaps, MT,
                                                            F, 2 * nmaps, gr.r0, tw, p.d_twoff, wph, nzr);
        note_launch();
    }
}

void launch_ring_analysis(const Plan &p, const double *maps, int64_t nmaps, double *F, cudaStream_t st, int *nzr) {
    if (p.precision == SFB_MIXED)
        ring_analysis_t<float, float, float2>(p, (const float *)maps, nmaps, (float *)F, p.d_twtab32, p.d_wphase32, st);
    else
        ring_analysis_t<double, double, double2>(p, maps, nmaps, F, p.d_twtab, p.d_wphase, st, nzr);
}

void launch_ring_synthesis(const Plan &p, const double *G, int64_t nmaps, double *maps, cudaStream_t st) {
    const int ns = (int)p.nside;
    const bool pow2 = (ns & (ns - 1)) == 0;
    struct Group { int r0, nr; size_t n; bool two; } groups[2] = {
        {0, ns - 1, (size_t)(4 * (ns - 1)), true},
        {ns - 1, ns + 1, (size_t)(4 * ns), !pow2}};
    for (const Group &gr : groups) {
        if (gr.nr <= 0) continue;
        const int MT = ring_mt(gr.n, sizeof(cx<double>), gr.two);
        const size_t smem = ring_smem(gr.n, sizeof(cx<double>), gr.two, MT);
        set_smem(k_ring_synthesis<double>, smem);
        dim3 grid((unsigned)gr.nr, (unsigned)((nmaps + MT - 1) / MT));
        k_ring_synthesis<double><<<grid, 256, smem, st>>>(p.d_rings, (int)p.nrn, p.lmax, G, 2 * nmaps, nmaps, MT,
                                                          p.npix, maps, gr.r0, p.d_twtab, p.d_twoff, p.d_phase);
        note_launch();
    }
}

}  // namespace sfb
