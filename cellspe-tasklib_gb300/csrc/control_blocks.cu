// The reference's Cell control blocks on the GPU (include/cellspe_control_blocks.h):
//  * cellspe_minicorrelator_run: the minicorrelator's SPE job for the six
//    `control_block`s of its 6-station setup (minicorrelator_spu.c:255-481),
//    as one FX correlation per output block on the engine, results scattered
//    to the reference's per-SPE autocorrelation and baseline-slot buffers;
//  * cellspe_cell_spectrometer_task: the Cell spectrometer's SPE task for one
//    `control_block_t` (spectrometer_spu.c:96-205): decode + window kernel,
//    batched real FFT, and a power kernel that carries the partly integrated
//    spectrum between tasks as the SPE keeps it in its local store.
#include "cellspe_control_blocks.h"
#include "cellspe_gpu.h"
#include "common.cuh"
#include "kernels.h"

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <vector>

namespace {

// ---------------------------------------------------------------------------
// minicorrelator
// ---------------------------------------------------------------------------
constexpr int MC_SPES = 6, MC_SLOTS = 15, MC_N = 2048, MC_C = 1024;
constexpr int MC_BYTES_PER_FFT = 256;           // one 1024-sample FFT buffer of 2-bit samples
constexpr int MC_PARTNER[3] = {1, 3, 4};        // minicorrelator_spu.c:302-304

#define CB_TRY(expr)                                                                   \
    do {                                                                               \
        cudaError_t _e = (expr);                                                       \
        if (_e != cudaSuccess) return cs_set_error(CELLSPE_ERR_CUDA, cudaGetErrorString(_e)); \
    } while (0)

int mc_fail(const char* msg) { return cs_set_error(CELLSPE_ERR_ARG, msg); }

// ---------------------------------------------------------------------------
// Cell spectrometer
// ---------------------------------------------------------------------------
struct CellSpec {
    int N = 0, K = 0, spr = 1;
    float levels[4] = {0, 0, 0, 0};
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    float* win = nullptr;          // [N] sin^2(pi i / (N - 1))
    float* acc = nullptr;          // [N/2 + 1] running spectrum
    int nacc = 0;                  // FFTs in the running spectrum
    uint8_t* raw = nullptr;        // chunk of raw bytes
    float* frames = nullptr;       // [chunk][N] windowed samples
    float2* bins = nullptr;        // [chunk][N/2 + 1]
    float* spectra = nullptr;      // [chunk spectra][2N] output staging
    int chunk = 0;                 // FFTs per chunk
    size_t raw_cap = 0;
};

void cellspec_free(CellSpec* s)
{
    if (!s) return;
    if (s->st) cudaStreamSynchronize(s->st);
    cudaFree(s->win);
    cudaFree(s->acc);
    cudaFree(s->raw);
    cudaFree(s->frames);
    cudaFree(s->bins);
    cudaFree(s->spectra);
    if (s->e0) cudaEventDestroy(s->e0);
    if (s->e1) cudaEventDestroy(s->e1);
    if (s->st) cudaStreamDestroy(s->st);
    delete s;
}

// windowed samples of FFT f (raw chunk starts at the chunk's first FFT)
__global__ void k_cellspec_frames(const uint8_t* __restrict__ raw, int N, int spr, int64_t d, int nf,
                                  const float* __restrict__ win, float4 lv, float* __restrict__ frames)
{
    const int64_t total = (int64_t)nf * N;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int f = (int)(t / N), i = (int)(t - (int64_t)f * N);
        float v;
        if (spr == 1) {
            v = (float)raw[f * d + i] - 127.5f;     // unpack_windowed_to_fft: byte - 127.5
        } else {
            const int code = (raw[f * d + (i >> 2)] >> (2 * (i & 3))) & 3;
            v = code == 0 ? lv.x : code == 1 ? lv.y : code == 2 ? lv.z : lv.w;
        }
        frames[t] = v * win[i];
    }
}

// One thread per bin k <= N/2: the chunk's FFT powers |X_k|^2 / K added in
// order; each time the running count reaches K the spectrum goes to output
// slot `done` as N {power, 0} pairs (bins k and N - k) and restarts at zero.
__global__ void k_cellspec_power(const float2* __restrict__ bins, int N, int K, int nf, int nacc0,
                                 float* __restrict__ acc, float* __restrict__ spectra)
{
    const int nb = N / 2 + 1;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nb) return;
    const float invK = 1.0f / (float)K;
    float a = acc[k];
    int n = nacc0, done = 0;
    for (int f = 0; f < nf; f++) {
        const float2 x = bins[(int64_t)f * nb + k];
        a += (x.x * x.x + x.y * x.y) * invK;
        if (++n == K) {
            float* out = spectra + (int64_t)done * 2 * N;
            out[2 * k] = a;
            out[2 * k + 1] = 0.f;
            if (k > 0 && k < N / 2) {
                out[2 * (N - k)] = a;
                out[2 * (N - k) + 1] = 0.f;
            }
            a = 0.f;
            n = 0;
            done++;
        }
    }
    acc[k] = a;
}

int cellspec_create(const control_block_t* cb, const float* levels4, CellSpec** out)
{
    const int N = (int)cb->fft_points;
    if (N < 32 || N > 32768 || (N & (N - 1)))
        return cs_set_error(CELLSPE_ERR_ARG, "cell_spectrometer_task: fft_points must be a power of two in [32, 32768]");
    if (cb->integrate_ffts == 0)
        return cs_set_error(CELLSPE_ERR_ARG, "cell_spectrometer_task: integrate_ffts must be > 0");
    if (cb->samples_per_rawbyte != 1 && cb->samples_per_rawbyte != 4)
        return cs_set_error(CELLSPE_ERR_ARG, "cell_spectrometer_task: samples_per_rawbyte must be 1 (8-bit) or 4 (2-bit)");
    auto* s = new CellSpec();
    s->N = N;
    s->K = (int)cb->integrate_ffts;
    s->spr = (int)cb->samples_per_rawbyte;
    if (levels4) std::memcpy(s->levels, levels4, sizeof s->levels);
    else cs_pick_levels(CELLSPE_LEVELS_TWOBIT, nullptr, s->levels);
    s->chunk = std::max(1, (1 << 22) / N);
    std::vector<float> w(N);
    for (int i = 0; i < N; i++) {
        const double v = std::sin(M_PI * (double)i / (double)(N - 1));
        w[i] = (float)(v * v);
    }
    const int nb = N / 2 + 1;
    const int max_spectra = s->chunk / s->K + 2;
    cudaError_t e = cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&s->e0);
    if (e == cudaSuccess) e = cudaEventCreate(&s->e1);
    if (e == cudaSuccess) e = cudaMalloc(&s->win, (size_t)N * 4);
    if (e == cudaSuccess) e = cudaMalloc(&s->acc, (size_t)nb * 4);
    if (e == cudaSuccess) e = cudaMalloc(&s->frames, (size_t)s->chunk * N * 4);
    if (e == cudaSuccess) e = cudaMalloc(&s->bins, (size_t)s->chunk * nb * 8);
    if (e == cudaSuccess) e = cudaMalloc(&s->spectra, (size_t)max_spectra * 2 * N * 4);
    // on the task's own (non-blocking) stream, ahead of its first kernels
    if (e == cudaSuccess) e = cudaMemcpyAsync(s->win, w.data(), (size_t)N * 4, cudaMemcpyHostToDevice, s->st);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->acc, 0, (size_t)nb * 4, s->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->st);
    if (e != cudaSuccess) {
        cellspec_free(s);
        return cs_set_error(CELLSPE_ERR_CUDA, cudaGetErrorString(e));
    }
    *out = s;
    return 0;
}

}  // namespace

extern "C" {

int cellspe_minicorrelator_run(const control_block* cbs, int num_spes)
{
    if (!cbs || num_spes != MC_SPES)
        return mc_fail("minicorrelator_run: needs the 6 control blocks of the reference's 6-station setup");
    const unsigned total = cbs[0].ffts_total, integ = cbs[0].ffts_to_integrate;
    const control_block* by_rank[MC_SPES] = {};
    for (int i = 0; i < MC_SPES; i++) {
        const control_block& c = cbs[i];
        if (c.ffts_total != total || c.ffts_to_integrate != integ)
            return mc_fail("minicorrelator_run: ffts_total and ffts_to_integrate differ between control blocks");
        if (c.spe_num < 0 || c.spe_num >= MC_SPES || by_rank[c.spe_num])
            return mc_fail("minicorrelator_run: spe_num must be a permutation of 0..5");
        by_rank[c.spe_num] = &c;
        if (!c.rawdata_src.p || !c.autocorrelation_out.p)
            return mc_fail("minicorrelator_run: null rawdata_src or autocorrelation_out");
        for (int m = 0; m < 3; m++)
            if (c.spe_num + MC_SPES * m < MC_SLOTS && !c.baselines_out[c.spe_num + MC_SPES * m].p)
                return mc_fail("minicorrelator_run: null baselines_out slot of this SPE");
    }
    if (integ < 2 || integ % 2 || total < integ)
        return mc_fail("minicorrelator_run: ffts_to_integrate must be even, >= 2 and <= ffts_total");
    const long long bytes = (long long)total * MC_BYTES_PER_FFT;
    if (bytes % 16) return mc_fail("minicorrelator_run: ffts_total x 256 bytes must be a multiple of 16");
    const int K = (int)(integ / 2);                       // 2048-sample segments per block
    const int blocks = (int)(total / integ);              // blocks written (minicorrelator_spu.c:839)
    // the stations' bytes back to back on the device, copied once for all blocks
    const int P = MC_SPES * (MC_SPES + 1) / 2;
    std::vector<std::complex<float>> vis((size_t)P * MC_C);
    struct DevBuf {
        void* p = nullptr;
        ~DevBuf() { cudaFree(p); }
    } d_raw, d_vis;
    CB_TRY(cudaMalloc(&d_raw.p, (size_t)MC_SPES * bytes));
    CB_TRY(cudaMalloc(&d_vis.p, vis.size() * sizeof(vis[0])));
    for (int s = 0; s < MC_SPES; s++)
        CB_TRY(cudaMemcpy(static_cast<char*>(d_raw.p) + (size_t)s * bytes, by_rank[s]->rawdata_src.p, bytes,
                          cudaMemcpyHostToDevice));
    cellspe_fx_params p;
    std::memset(&p, 0, sizeof p);
    p.n_inputs = MC_SPES;
    p.fft_points = MC_N;
    p.n_segments = K;
    p.x_mode = CELLSPE_X_FP32;
    p.vis_order = CELLSPE_VIS_BASELINE_MAJOR;
    p.levels = CELLSPE_LEVELS_OFFSET_BINARY;
    p.bytes_per_input = bytes;
    p.memory = CELLSPE_MEM_DEVICE;
    auto tri = [](int i, int j) { return i * (i + 1) / 2 + j; };
    for (int b = 0; b < blocks; b++) {
        p.start_sample = (long long)b * K * MC_N;
        const int rc = cellspe_fx_correlate(&p, d_raw.p, nullptr, d_vis.p);   // returns when done
        if (rc) return rc;
        CB_TRY(cudaMemcpy(vis.data(), d_vis.p, vis.size() * sizeof(vis[0]), cudaMemcpyDeviceToHost));
        auto put = [&](void* dst, int i, int j, bool conj) {      // planar Re x 1024 | Im x 1024 of block b
            float* o = static_cast<float*>(dst) + (size_t)b * 2 * MC_C;
            const std::complex<float>* v = vis.data() + (size_t)tri(i, j) * MC_C;
            for (int c = 0; c < MC_C; c++) {
                o[c] = v[c].real();
                o[MC_C + c] = conj ? -v[c].imag() : v[c].imag();
            }
        };
        for (int s = 0; s < MC_SPES; s++) {
            const control_block& c = *by_rank[s];
            put(c.autocorrelation_out.p, s, s, false);
            for (int m = 0; m < 3; m++) {
                const int slot = s + MC_SPES * m;
                if (slot >= MC_SLOTS) continue;
                const int o = (s + MC_PARTNER[m]) % MC_SPES;
                // X_s conj(X_o): stored for s > o, its conjugate otherwise
                if (s > o) put(c.baselines_out[slot].p, s, o, false);
                else put(c.baselines_out[slot].p, o, s, true);
            }
        }
    }
    return 0;
}

int cellspe_cell_spectrometer_task(void** state, const control_block_t* cb, const float* levels4, unsigned int stats[3])
{
    if (!state || !cb) return cs_set_error(CELLSPE_ERR_ARG, "cell_spectrometer_task: null state or control block");
    if (stats) stats[0] = stats[1] = stats[2] = 0;
    if (cb->terminate_flag) {                             // spectrometer_spu.c:122-125
        cellspec_free(static_cast<CellSpec*>(*state));
        *state = nullptr;
        return 0;
    }
    if (!*state) {                                        // preinit (spectrometer_spu.c:128-155)
        CellSpec* s = nullptr;
        const int rc = cellspec_create(cb, levels4, &s);
        if (rc) return rc;
        *state = s;
    }
    CellSpec& s = *static_cast<CellSpec*>(*state);
    const int N = s.N, nb = N / 2 + 1;
    const int64_t rb = N / s.spr;                         // raw bytes of one FFT
    if (cb->overlap_factor == 0 || rb / cb->overlap_factor == 0)
        return cs_set_error(CELLSPE_ERR_ARG, "cell_spectrometer_task: overlap_factor must be in [1, raw bytes per FFT]");
    const int64_t d = rb / cb->overlap_factor;            // raw_delta_bytelen
    const int64_t B = cb->rawif_bytecount;
    int64_t nfft = B >= 2 * d ? B / d - 1 : 0;            // the SPE's loop count
    nfft = std::min<int64_t>(nfft, B >= rb ? (B - rb) / d + 1 : 0);   // no FFT past the buffer
    if (nfft > 0 && !cb->rawif_src.p) return cs_set_error(CELLSPE_ERR_ARG, "cell_spectrometer_task: null rawif_src");
    if (nfft + s.nacc >= s.K && !cb->spectrum_dst.p)
        return cs_set_error(CELLSPE_ERR_ARG, "cell_spectrometer_task: null spectrum_dst");
    const auto* src = static_cast<const uint8_t*>(cb->rawif_src.p);
    float* dst = static_cast<float*>(cb->spectrum_dst.p);
    CB_TRY(cudaEventRecord(s.e0, s.st));
    unsigned spectra = 0;
    const float4 lv = make_float4(s.levels[0], s.levels[1], s.levels[2], s.levels[3]);
    for (int64_t f0 = 0; f0 < nfft; f0 += s.chunk) {
        const int nf = (int)std::min<int64_t>(s.chunk, nfft - f0);
        const size_t bytes = (size_t)((nf - 1) * d + rb);
        if (bytes > s.raw_cap) {
            CB_TRY(cudaStreamSynchronize(s.st));
            cudaFree(s.raw);
            s.raw = nullptr;
            s.raw_cap = 0;
            CB_TRY(cudaMalloc(&s.raw, bytes));
            s.raw_cap = bytes;
        }
        CB_TRY(cudaMemcpyAsync(s.raw, src + f0 * d, bytes, cudaMemcpyHostToDevice, s.st));
        const int64_t total = (int64_t)nf * N;
        const int grid = (int)std::min<int64_t>((total + 255) / 256, 152 * 16);
        k_cellspec_frames<<<grid, 256, 0, s.st>>>(s.raw, N, s.spr, d, nf, s.win, lv, s.frames), cs_count_launches(1);
        int rc = cs_rfft_batch(s.frames, s.bins, N, nf, s.st);
        if (rc) return cs_set_error(CELLSPE_ERR_CUDA, "cell_spectrometer_task: batched FFT failed");
        k_cellspec_power<<<(nb + 255) / 256, 256, 0, s.st>>>(s.bins, N, s.K, nf, s.nacc, s.acc, s.spectra),
            cs_count_launches(1);
        CB_TRY(cudaGetLastError());
        const int done = (s.nacc + nf) / s.K;
        s.nacc = (s.nacc + nf) % s.K;
        if (done) {
            CB_TRY(cudaMemcpyAsync(dst + (size_t)spectra * 2 * N, s.spectra, (size_t)done * 2 * N * 4,
                                   cudaMemcpyDeviceToHost, s.st));
            spectra += done;
        }
        CB_TRY(cudaStreamSynchronize(s.st));              // the raw chunk and the staging are reused
    }
    CB_TRY(cudaEventRecord(s.e1, s.st));
    CB_TRY(cudaEventSynchronize(s.e1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, s.e0, s.e1);
    if (stats) {
        const double ns = (double)ms * 1e6;
        stats[0] = ns > 4294967295.0 ? 0xFFFFFFFFu : (unsigned)ns;
        stats[1] = spectra;
        stats[2] = (unsigned)nfft;
    }
    return 0;
}

}  // extern "C"
