// sfb_winweights2galweights_noalloc: the per-galaxy weight gather of
// sfb_winweights2galweights, staged through a fixed device array instead of
// memory allocated per call.
//
// Who needs it: a caller whose device memory is owned by someone else's pool
// (a Julia or PyTorch caching allocator that has reserved nearly all of HBM),
// or that runs where a new allocation is not allowed (cudaMalloc/cudaFree
// synchronise the whole device and can fail under memory pressure part way
// through a pipeline).  Such a caller cannot use the ordinary entry point,
// which allocates its staging buffers on every call.
//
// Scratch: one static array of SCRATCH_DOUBLES doubles (16 MiB) per device
// and process, laid out as
//   [error word: HEAD doubles][weights nr*npix][rbounds nr+1][galaxy chunk: 3 rtp + 1 w each]
// The weight table must fit in the array with room for MIN_CHUNK galaxies;
// larger tables are rejected with SFB_EINVAL.  Galaxies stream through the
// remaining space in chunks.  Only the error word has to start at zero; each
// call clears it before its first launch.  Every other element is written by
// a copy before any kernel reads it.
//
// Set-up: the first call on a device (with that device current) looks up the
// array's device address with cudaGetSymbolAddress; this loads the library's
// device code on that device.  Make that first call before any stream capture.
// The address is kept for the life of the process: a cudaDeviceReset of the
// device invalidates it, and a process that resets a device must not call this
// entry point on it again.
//
// Streams: every copy and the kernel go to the legacy default stream with
// synchronous cudaMemcpy, so the call returns with its result on the host and
// serialises with every blocking stream of the process.
//
// Overlapping calls on one device would race on the single scratch array; the
// calls are serialised by a per-device lock, so concurrent callers on one
// device wait for each other.  Separate processes have separate arrays.

#include "sfb_internal.h"

#include <mutex>
#include <string>

namespace sfb {
// the gather kernel of sfb_winweights2galweights (radial.cu)
void launch_winweights(const double *weights, int64_t nr, int64_t nside, const double *rbounds, double rmax,
                       const double *rtp, int64_t ngal, double *w, int *err, cudaStream_t st);
}  // namespace sfb

using namespace sfb;

namespace {

constexpr int64_t SCRATCH_DOUBLES = int64_t(1) << 21;  // 16 MiB
constexpr int64_t HEAD = 32;                           // 256 bytes for the error word
constexpr int64_t MIN_CHUNK = 4096;                    // galaxies per staged chunk, at least
constexpr int64_t MAX_TABLE = SCRATCH_DOUBLES - HEAD - 4 * MIN_CHUNK;
constexpr int MAX_DEVICES = 64;

__device__ __align__(256) double g_ww_scratch[SCRATCH_DOUBLES];

std::mutex g_setup_mu;
std::mutex g_call_mu[MAX_DEVICES];
double *g_scratch_of[MAX_DEVICES] = {};

// Device address of g_ww_scratch on the current device (looked up once).
int scratch_for_current_device(int *dev_out, double **out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(SFB_ECUDA, std::string("no CUDA device: ") + cudaGetErrorString(e));
    }
    if (dev < 0 || dev >= MAX_DEVICES) return fail(SFB_ENOTSUP, "device ordinal beyond 63");
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_scratch_of[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_ww_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return fail(SFB_ECUDA, std::string("static scratch lookup failed: ") + cudaGetErrorString(e));
        }
        g_scratch_of[dev] = static_cast<double *>(p);
    }
    *dev_out = dev;
    *out = g_scratch_of[dev];
    return SFB_OK;
}

}  // namespace

extern "C" int sfb_winweights2galweights_noalloc(int64_t nside, const double *weights, int64_t nr,
                                                 const double *rbounds, const double *rtp, int64_t ngal,
                                                 double *w_out) {
    if (nside < 1 || nr < 1 || !weights || !rbounds || ngal < 0 || (ngal > 0 && (!rtp || !w_out)))
        return fail(SFB_EINVAL, "bad winweights2galweights arguments");
    if (ngal == 0) return SFB_OK;
    if (nside > (int64_t(1) << 13) || nr > MAX_TABLE)
        return fail(SFB_EINVAL, "winweights table beyond the static scratch maximum of " +
                                    std::to_string(MAX_TABLE) + " doubles");
    const int64_t npix = 12 * nside * nside;
    const int64_t table = nr * npix + nr + 1;
    if (nr > MAX_TABLE / npix || table > MAX_TABLE)
        return fail(SFB_EINVAL, "winweights table of nr*npix + nr + 1 = " + std::to_string(nr) + "*" +
                                    std::to_string(npix) + " + " + std::to_string(nr + 1) +
                                    " doubles exceeds the static scratch maximum of " + std::to_string(MAX_TABLE) +
                                    " doubles");
    int dev = -1;
    double *s = nullptr;
    SFB_TRY(scratch_for_current_device(&dev, &s));
    std::lock_guard<std::mutex> lock(g_call_mu[dev]);

    int *derr = reinterpret_cast<int *>(s);
    double *dw = s + HEAD;
    double *db = dw + nr * npix;
    double *dgal = db + nr + 1;
    const int64_t chunk = (SCRATCH_DOUBLES - HEAD - table) / 4;
    double *dr = dgal;
    double *dout = dgal + 3 * chunk;

    auto cuda_fail = [](cudaError_t e) {
        cudaGetLastError();
        return fail(SFB_ECUDA, cudaGetErrorString(e));
    };
    cudaError_t e;
    if ((e = cudaMemset(derr, 0, sizeof(int))) != cudaSuccess) return cuda_fail(e);
    if ((e = cudaMemcpy(dw, weights, sizeof(double) * nr * npix, cudaMemcpyHostToDevice)) != cudaSuccess)
        return cuda_fail(e);
    if ((e = cudaMemcpy(db, rbounds, sizeof(double) * (nr + 1), cudaMemcpyHostToDevice)) != cudaSuccess)
        return cuda_fail(e);
    for (int64_t g0 = 0; g0 < ngal; g0 += chunk) {
        const int64_t n = (ngal - g0 < chunk) ? ngal - g0 : chunk;
        if ((e = cudaMemcpy(dr, rtp + 3 * g0, sizeof(double) * 3 * n, cudaMemcpyHostToDevice)) != cudaSuccess)
            return cuda_fail(e);
        launch_winweights(dw, nr, nside, db, rbounds[nr], dr, n, dout, derr, 0);
        if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e);
        if ((e = cudaMemcpy(w_out + g0, dout, sizeof(double) * n, cudaMemcpyDeviceToHost)) != cudaSuccess)
            return cuda_fail(e);
    }
    int herr = 0;
    if ((e = cudaMemcpy(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost)) != cudaSuccess) return cuda_fail(e);
    if (herr & ERR_NONFINITE_INPUT) return fail(SFB_ENONFINITE, "non-finite galaxy coordinate");
    if (herr & ERR_RANGE_R) return fail(SFB_ERANGE, "r out of bounds");
    return SFB_OK;
}
