// Ring geometry, associated-Legendre table, and small utility kernels.
#include "sfb_internal.h"

namespace sfb {

// lambda_lm(theta_r) for every north ring r and m <= l <= lmax, FP64.
// Y_lm = lambda_lm e^{i m phi} with the Condon-Shortley phase (the convention
// of the reference's sphericalharmonicsy, src/math.jl:10-21).  One thread per
// (m, ring) runs the three-term recursion in l; a power-of-two exponent is
// carried so that lambda_mm ~ sin^m(theta) cannot underflow before the
// recursion in l grows it back.  Table block (m, parity) holds rows
// l = m + parity + 2*li, each row nrn rings long.
__global__ void k_legendre_table(const RingGeom *rings, int nrn, int lmax, const int64_t *lam_off,
                                 double *lam) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    const int m = blockIdx.y;
    if (r >= nrn || m > lmax) return;
    const double z = rings[r].z;
    const double sth = rings[r].sth;
    const double two600 = 4.149515568880993e+180;   // 2^600
    const double twom600 = 2.409919865102884e-181;  // 2^-600
    double mant = 0.28209479177387814347;           // 1/sqrt(4 pi)
    int e = 0;
    for (int k = 1; k <= m; ++k) {
        mant = mant * (-sqrt((2.0 * k + 1.0) / (2.0 * k))) * sth;
        if (fabs(mant) < twom600 && mant != 0.0) {
            mant *= two600;
            e -= 600;
        }
    }
    double *blk0 = lam + lam_off[2 * m];
    double *blk1 = lam + lam_off[2 * m + 1];
    blk0[r] = ldexp(mant, e);  // l = m, parity 0, li = 0
    double prev2 = 0.0, prev = mant;
    for (int l = m + 1; l <= lmax; ++l) {
        const double a = sqrt((4.0 * l * l - 1.0) / ((double)l * l - (double)m * m));
        const double b = (l - 1 > m) ? sqrt(((double)(l - 1) * (l - 1) - (double)m * m) /
                                            (4.0 * (l - 1) * (l - 1) - 1.0))
                                     : 0.0;
        double v = a * (z * prev - b * prev2);
        if (fabs(v) > two600) {
            v *= twom600;
            prev *= twom600;
            e += 600;
        }
        const int par = (l - m) & 1;
        const int li = (l - m - par) >> 1;
        (par ? blk1 : blk0)[(int64_t)li * nrn + r] = ldexp(v, e);
        prev2 = prev;
        prev = v;
    }
}

void launch_legendre_table(const Plan &p, cudaStream_t st) {
    dim3 grid((unsigned)((p.nrn + 127) / 128), (unsigned)(p.lmax + 1));
    k_legendre_table<<<grid, 128, 0, st>>>(p.d_rings, (int)p.nrn, p.lmax, p.d_lam_off, p.d_lam);
    note_launch();
}

__global__ void k_ang2pix(int64_t nside, const double *theta, const double *phi, int64_t n, int64_t *pix) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    pix[i] = ang2pix_ring_fast(nside, theta[i], phi[i]);
}

void launch_ang2pix(int64_t nside, const double *theta, const double *phi, int64_t n, int64_t *pix,
                    cudaStream_t st) {
    if (n <= 0) return;
    k_ang2pix<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(nside, theta, phi, n, pix);
    note_launch();
}

// out[c][r] = in[r][c]; in is rows x cols row-major.
__global__ void k_transpose(const double *in, int64_t rows, int64_t cols, double *out) {
    __shared__ double tile[32][33];
    const int64_t c0 = (int64_t)blockIdx.x * 32;
    for (int64_t r0 = (int64_t)blockIdx.y * 32; r0 < rows; r0 += (int64_t)gridDim.y * 32) {   // grid y <= 65535
        for (int j = threadIdx.y; j < 32; j += 8) {
            const int64_t r = r0 + j, c = c0 + threadIdx.x;
            if (r < rows && c < cols) tile[j][threadIdx.x] = in[r * cols + c];
        }
        __syncthreads();
        for (int j = threadIdx.y; j < 32; j += 8) {
            const int64_t c = c0 + j, r = r0 + threadIdx.x;
            if (r < rows && c < cols) out[c * rows + r] = tile[threadIdx.x][j];
        }
        __syncthreads();
    }
}

void launch_transpose(const double *in, int64_t rows, int64_t cols, double *out, cudaStream_t st) {
    if (rows <= 0 || cols <= 0) return;
    dim3 grid((unsigned)((cols + 31) / 32), (unsigned)std::min<int64_t>((rows + 31) / 32, 65535));
    k_transpose<<<grid, dim3(32, 8), 0, st>>>(in, rows, cols, out);
    note_launch();
}

__device__ __forceinline__ float2 convert_elem(float v, float2 *) { return make_float2(v, 0.f); }
template <typename TI, typename TO>
__device__ __forceinline__ TO convert_elem(TI v, TO *) { return (TO)v; }

// out[c * ldo + r] = in[r * ldi + c] for r < rows, c < cols (converted to TO; float -> double-float
// pairs with a zero low word).
template <typename TI, typename TO>
__global__ void k_transpose_ld(const TI *in, int64_t ldi, int64_t rows, int64_t cols, TO *out, int64_t ldo) {
    __shared__ TI tile[32][33];
    const int64_t c0 = (int64_t)blockIdx.x * 32;
    // row tiles over grid y, which is capped at 65535 (rows are pixels: 98304 tiles at nside 512)
    for (int64_t r0 = (int64_t)blockIdx.y * 32; r0 < rows; r0 += (int64_t)gridDim.y * 32) {
        for (int j = threadIdx.y; j < 32; j += 8) {
            const int64_t r = r0 + j, c = c0 + threadIdx.x;
            if (r < rows && c < cols) tile[j][threadIdx.x] = in[r * ldi + c];
        }
        __syncthreads();
        for (int j = threadIdx.y; j < 32; j += 8) {
            const int64_t c = c0 + j, r = r0 + threadIdx.x;
            if (r < rows && c < cols) out[c * ldo + r] = convert_elem(tile[threadIdx.x][j], (TO *)nullptr);
        }
        __syncthreads();
    }
}

template <typename TI, typename TO>
static void transpose_ld(const TI *in, int64_t ldi, int64_t rows, int64_t cols, TO *out, int64_t ldo,
                         cudaStream_t st) {
    if (rows <= 0 || cols <= 0) return;
    dim3 grid((unsigned)((cols + 31) / 32), (unsigned)std::min<int64_t>((rows + 31) / 32, 65535));
    k_transpose_ld<TI, TO><<<grid, dim3(32, 8), 0, st>>>(in, ldi, rows, cols, out, ldo);
    note_launch();
}

void launch_transpose_ld(const double *in, int64_t ldi, int64_t rows, int64_t cols, double *out, int64_t ldo,
                         cudaStream_t st) {
    transpose_ld(in, ldi, rows, cols, out, ldo, st);
}
void launch_transpose_ld(const float *in, int64_t ldi, int64_t rows, int64_t cols, double *out, int64_t ldo,
                         cudaStream_t st) {
    transpose_ld(in, ldi, rows, cols, out, ldo, st);
}
void launch_transpose_ld(const float *in, int64_t ldi, int64_t rows, int64_t cols, float *out, int64_t ldo,
                         cudaStream_t st) {
    transpose_ld(in, ldi, rows, cols, out, ldo, st);
}
void launch_transpose_ld(const double *in, int64_t ldi, int64_t rows, int64_t cols, float *out, int64_t ldo,
                         cudaStream_t st) {
    transpose_ld(in, ldi, rows, cols, out, ldo, st);
}
void launch_transpose_ld(const float *in, int64_t ldi, int64_t rows, int64_t cols, float2 *out, int64_t ldo,
                         cudaStream_t st) {
    transpose_ld(in, ldi, rows, cols, out, ldo, st);
}

__global__ void k_check_finite(const double *x, int64_t n, int *err) {
    int bad = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        if (!isfinite(x[i])) bad = 1;
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(err, ERR_NONFINITE_OUTPUT);
}

void launch_check_finite(const double *x, int64_t n, int *err, cudaStream_t st) {
    if (n <= 0) return;
    int64_t blocks = (n + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    k_check_finite<<<(unsigned)blocks, 256, 0, st>>>(x, n, err);
    note_launch();
}

}  // namespace sfb
