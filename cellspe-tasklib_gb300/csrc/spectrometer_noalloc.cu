// Spectrometer entry point that allocates no device memory.
//
// Some callers cannot call cudaMalloc at the time they run the spectrometer:
// real-time capture loops that must not block on the allocator (cudaMalloc
// and cudaFree can synchronise the whole device), code that runs while a CUDA
// graph is being captured, or hosts that hand this library a fixed device
// budget up front and forbid any later allocation.  cellspe_spectrometer
// stages its chunk partial spectra and phase-cal partials in a workspace
// that it allocates on demand; this variant uses the fixed arrays below
// instead, so the caller only provides the input planes and the outputs.
//
// Limits and behaviour:
// * The arrays live in this library's static device memory: every GPU that
//   loads the library holds them (about 17.3 MiB) until the process exits.
// * Partial spectra get at most CS_NOALLOC_SCRATCH_FLOATS floats (16 MiB).
//   The FFTs of a spectrum are grouped into as few chunks as needed to fit;
//   jobs that do not fit even with one chunk per spectrum are rejected.
// * FFT size, window and phase-cal rotator tables are rebuilt by small
//   kernels on the caller's stream on every call (no host-side caching).
// * Every scratch element a call reads was written earlier in that call, so
//   nothing needs clearing between calls; calls whose work overlaps on the
//   GPU (different streams, or different host threads) share the arrays and
//   race.
// * The first call on a device looks up the arrays' device addresses with
//   cudaGetSymbolAddress (host code may not use a __device__ symbol's name
//   as a device pointer); make that first call before any stream capture.
#include "../../include/cellspe_gpu.h"
#include "common.cuh"
#include "kernels.h"

#include <cmath>
#include <mutex>

namespace {

constexpr size_t CS_NOALLOC_SCRATCH_FLOATS = (size_t)4 << 20;    // 16 MiB of partials
constexpr int CS_NOALLOC_MAX_N = 65536;

static __device__ __align__(256) float g_noalloc_scratch[CS_NOALLOC_SCRATCH_FLOATS];
static __device__ __align__(256) float2 g_noalloc_tw[CS_NOALLOC_MAX_N];
static __device__ __align__(256) float g_noalloc_win[CS_NOALLOC_MAX_N];
static __device__ __align__(256) float2 g_noalloc_rot[CS_NOALLOC_MAX_N];

struct NoallocPtrs {
    float* scratch = nullptr;
    float2* tw = nullptr;
    float* win = nullptr;
    float2* rot = nullptr;
    bool ready = false;
};
constexpr int MAX_DEVICES = 64;
std::mutex g_setup_mu;
NoallocPtrs g_ptrs[MAX_DEVICES];

int setup_device(int dev, NoallocPtrs* out)
{
    if (dev < 0 || dev >= MAX_DEVICES) return CELLSPE_ERR_UNSUPPORTED;
    std::lock_guard<std::mutex> lk(g_setup_mu);
    NoallocPtrs& p = g_ptrs[dev];
    if (!p.ready) {
        cudaError_t e = cudaGetSymbolAddress((void**)&p.scratch, g_noalloc_scratch);
        if (e == cudaSuccess) e = cudaGetSymbolAddress((void**)&p.tw, g_noalloc_tw);
        if (e == cudaSuccess) e = cudaGetSymbolAddress((void**)&p.win, g_noalloc_win);
        if (e == cudaSuccess) e = cudaGetSymbolAddress((void**)&p.rot, g_noalloc_rot);
        if (e != cudaSuccess) return cs_set_error(CELLSPE_ERR_CUDA, "spectrometer_noalloc: cudaGetSymbolAddress failed");
        p.ready = true;
    }
    *out = p;
    return 0;
}

// The host-built tables of the allocating path, by the same FP64 formulas
// rounded to FP32 (the device's FP64 cos/sin may differ from the host's in
// the last bit of a double, which can move a rounded entry by one FP32 ulp).
__global__ void k_fill_tables(float2* tw, float* win, int n, int window, float2* rot, int rotlen, double dphi)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const double a = -2.0 * M_PI * (double)i / (double)n;
        tw[i] = make_float2((float)cos(a), (float)sin(a));
        win[i] = (float)cs_window_value(window, i, n);
    }
    if (i < rotlen) rot[i] = make_float2((float)cos(dphi * (double)i), (float)sin(dphi * (double)i));
}

}  // namespace

extern "C" int cellspe_spectrometer_noalloc(const cellspe_spec_params* p, const void* raw, float* power,
                                            void* pcal_bins, void* pcal_tones, void* stream)
{
    if (!p || !raw || !power) return cs_set_error(CELLSPE_ERR_ARG, "spectrometer_noalloc: null argument");
    // the checks cellspe_spectrometer runs, then the limits of this entry point
    if (int rc = cs_spec_check(p, "spectrometer_noalloc")) return rc;
    if (p->memory != CELLSPE_MEM_DEVICE)
        return cs_set_error(CELLSPE_ERR_ARG, "spectrometer_noalloc: device memory only (memory = CELLSPE_MEM_DEVICE)");
    const int nsub = p->n_subbands;
    if (p->input_layout == CELLSPE_SPEC_MARK5B_FRAMED || p->input_layout == CELLSPE_SPEC_VDIF_FRAMED)
        return cs_set_error(CELLSPE_ERR_ARG, "spectrometer_noalloc: framed input needs deframing scratch");
    if (nsub > 1 && p->input_layout != CELLSPE_SPEC_PLANES)
        return cs_set_error(CELLSPE_ERR_ARG,
                            "spectrometer_noalloc: needs CELLSPE_SPEC_PLANES input (the corner turn needs a raw-sized buffer)");
    const int N = p->fft_points;
    if (p->pcal_tonebins > 0 && (!pcal_bins || p->pcal_rotatorlen <= 0 || p->pcal_rotatorlen > CS_NOALLOC_MAX_N))
        return cs_set_error(CELLSPE_ERR_ARG, "spectrometer_noalloc: phase-cal needs pcal_bins and rotatorlen <= 65536");
    float lut[4];
    if (!cs_pick_levels(p->levels, p->custom_levels, lut))
        return cs_set_error(CELLSPE_ERR_ARG, "spectrometer_noalloc: unknown level table");

    // Chunking: the default number of FFTs per partial, grown until the
    // partials (plus phase-cal partials) fit the static scratch.
    CsSpecArgs a{};
    a.planes = (const uint8_t*)raw;
    a.bytes_per_sub = p->raw_bytes / nsub;
    a.nsub = nsub; a.N = N; a.overlap = p->overlap; a.window = p->window;
    a.ffts_per_spectrum = p->ffts_per_spectrum; a.nspec = p->n_spectra;
    for (int i = 0; i < 4; i++) a.lut[i] = lut[i];
    a.tonebins = p->pcal_tonebins; a.rotatorlen = p->pcal_rotatorlen; a.ntones = p->pcal_ntones;
    a.pcal_offset_hz = p->pcal_offset_hz; a.fs_hz = p->sample_rate_hz;
    a.power = power;
    a.pcal_bins = (float2*)pcal_bins;
    a.pcal_tones = (float2*)pcal_tones;
    const long long novl = (long long)p->overlap * p->ffts_per_spectrum - (p->overlap - 1);
    a.ffts_per_chunk = 0;
    if ((size_t)cs_spectrometer_scratch_floats(a) > CS_NOALLOC_SCRATCH_FLOATS) {
        const long long rows = (long long)nsub * p->n_spectra, nb = N / 2 + 1;
        // phase-cal partials + 64 floats of alignment between the two parts
        const long long pcal = cs_spectrometer_pcal_floats(a) + 64;
        const long long max_chunks = ((long long)CS_NOALLOC_SCRATCH_FLOATS - pcal) / (rows * nb);
        if (max_chunks < 1)
            return cs_set_error(CELLSPE_ERR_ARG,
                                "spectrometer_noalloc: job exceeds the static scratch maximum of 4194304 floats "
                                "((n_subbands * n_spectra) * (fft_points/2+1) must fit, plus phase-cal partials)");
        a.ffts_per_chunk = (int)((novl + max_chunks - 1) / max_chunks);
        if ((size_t)cs_spectrometer_scratch_floats(a) > CS_NOALLOC_SCRATCH_FLOATS)
            return cs_set_error(CELLSPE_ERR_ARG, "spectrometer_noalloc: job exceeds the static scratch maximum");
    }

    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return cs_set_error(CELLSPE_ERR_CUDA, "spectrometer_noalloc: no device");
    NoallocPtrs ptrs;
    int rc = setup_device(dev, &ptrs);
    if (rc) return rc;
    a.partial = ptrs.scratch;
    a.tw_table = ptrs.tw;
    a.win_table = ptrs.win;
    a.rot_table = ptrs.rot;

    cudaStream_t st = (cudaStream_t)stream;
    const int rotlen = p->pcal_tonebins > 0 ? p->pcal_rotatorlen : 0;
    const int nfill = N > rotlen ? N : rotlen;
    const double dphi = rotlen > 0 ? 2.0 * M_PI * (-p->pcal_offset_hz / p->sample_rate_hz) : 0.0;   // fs > 0 checked
    k_fill_tables<<<(nfill + 255) / 256, 256, 0, st>>>(ptrs.tw, ptrs.win, N, p->window, ptrs.rot, rotlen, dphi),
        cs_count_launches(1);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cs_set_error(CELLSPE_ERR_CUDA, "spectrometer_noalloc: table kernel launch failed");
    rc = cs_spectrometer(a, st);
    if (rc == CS_ERR_ARG) return cs_set_error(CELLSPE_ERR_ARG, "spectrometer_noalloc: invalid argument");
    if (rc == CS_ERR_UNSUPPORTED) return cs_set_error(CELLSPE_ERR_UNSUPPORTED, "spectrometer_noalloc: unsupported size");
    if (rc) return cs_set_error(CELLSPE_ERR_CUDA, "spectrometer_noalloc: kernel launch failed");
    return 0;
}
