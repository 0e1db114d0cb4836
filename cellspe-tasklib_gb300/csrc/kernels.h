// Internal launch API between the C-ABI runtime (runtime.cpp) and the CUDA
// kernels.  Every launcher is asynchronous on the given stream and returns 0
// or a cudaError_t / CS_ERR_* code.  Pointers are device pointers.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/cellspe_gpu.h"

#define CS_ERR_ARG 10001      // invalid argument (size, alignment, null)
#define CS_ERR_UNSUPPORTED 10002

// Count of kernel launches issued by this library (read by the benchmark to
// report how many of its own kernels ran in a timed region).
long long cs_launch_count();
void cs_count_launches(int n);
// Records the calling thread's error text for cellspe_last_error(); returns code.
int cs_set_error(int code, const char* msg);

// unpack.cu -----------------------------------------------------------------
int cs_unpack2bit(const void* raw, int64_t nsamp, int nchan, int msb_first, const float lut4[4],
                  float* out, cudaStream_t st);
int cs_cornerturn2bit(const void* raw, int64_t nsamp, int nchan, void* planes, cudaStream_t st);

// fft.cu --------------------------------------------------------------------
// Twiddle table exp(-2 pi i m / n), m in [0, n), FP64-computed, device copy.
// Cached per (device, n); valid until cs_free_twiddles().
const float2* cs_twiddles(int n);
// Raise (never lower) a kernel's dynamic shared-memory limit to `bytes`.
cudaError_t cs_smem_at_least(const void* fn, int bytes);
void cs_free_twiddles();
// Batched forward C2C FFT, n points (32..16384), interleaved complex.
int cs_cfft_batch(const float2* in, float2* out, int n, int64_t batch, cudaStream_t st);
// Batched backward C2C FFT (e^{+2 pi i nk/n}, FFTW_BACKWARD, unnormalised)
// with every output multiplied by `scale`.
int cs_cfft_inverse_batch(const float2* in, float2* out, int n, int64_t batch, float scale, cudaStream_t st);
// Batched forward R2C FFT, n real points (64..32768) -> n/2+1 bins.
int cs_rfft_batch(const float* in, float2* out, int n, int64_t batch, cudaStream_t st);
// Real-FFT bins [batch][n/2+1] -> IPP Perm rows [batch][n] floats
// ([R0, R_{n/2}, Re 1, Im 1, ...]).  bins and out must not overlap.
int cs_perm_pack(const float2* bins, float* out, int n, int64_t batch, cudaStream_t st);

// fstage.cu -----------------------------------------------------------------
struct CsDelayState {       // per (input, segment)
    int32_t* shift;         // integer sample shift
    float* phase0;          // fringe phase, radians in [0, 2 pi)
    float* dphase;          // per-channel phase step, radians
};
// FP64 delay model -> delay state.  poly: [S][4] seconds (t^0..t^3).
int cs_delay_state(const double* poly, int S, int N, int K, double fs_hz, double lo_hz,
                   CsDelayState ds, cudaStream_t st);

enum CsSpectraFormat { CS_SPECTRA_F32 = 0, CS_SPECTRA_F16 = 1 };
struct CsFStageArgs {
    const uint8_t* raw;         // [S][bytes_per_input], 2-bit single channel
    int64_t bytes_per_input;
    int S, N, K;
    int64_t start_sample;
    const int32_t* shift;       // [S*K] or null
    const float* phase0;        // [S*K] or null (no phase correction)
    const float* dphase;        // [S*K]
    const float* scale;         // [S*C] per (input, channel) scale or null (1.0)
    float lut[4];
    int msb_first;
    int format;                 // CsSpectraFormat
    void* out;                  // F32: float2 [C][S][kp];  F16: __half [C][2][S][kp]
    int kp;                     // row pitch of out in elements (>= K; 0 = K)
    int S_out;                  // inputs in the output layout (0 = S): a launch over a
                                // block of inputs writes at out + s0 * kp with rows
                                // (c, plane) S_out * kp apart
    int seg_major;              // 1: out is [S][K][C] (F32 float2, F16 half2 Re|Im), each
                                // segment's spectrum contiguous; cs_spectra_transpose then
                                // makes the channel-major layout (the generic kernels only)
    int kblock;                 // F16 only: 1 k-blocked rows, 2 channel-grouped k-blocked
                                // rows; see cs_fstage_layout
};
int cs_fx_fstage(const CsFStageArgs& a, cudaStream_t st);
// Per host thread: whether the 2048-point F stage may time its schedules on
// this thread's jobs (default true; the correlation service's workers turn it
// off and use the last timed schedule).
void cs_fstage_allow_timing(bool allow);
bool cs_fstage_timing_allowed();   // this thread may time kernel choices (autotuners)
// True when the F stage for these arguments writes FP16 spectra k-blocked:
// __half [C][S_out][kp/32][2][32], i.e. for each (channel, input) and block of
// 32 segments the 32 Re halves then the 32 Im halves (128 contiguous bytes, the
// 2048-point warp F stage's 32-segment tiles).  Needs N = 2048, K and kp
// multiples of 32; the X stage then reads the same layout (kblock = 1).  A
// launch over a block of inputs writes at out + s0 * kp * 4 bytes.
bool cs_fstage_kblocked(const CsFStageArgs& a);
// The spectra layout the F stage writes for these arguments (its kblock):
// 0 channel-major planes (or segment-major, see seg_major); 1 k-blocked as
// above; 2 channel-grouped k-blocked: the same 128-byte (32 Re, 32 Im) runs,
// ordered [C/16][S_out][kp/32][16]: run (c, s, b) at ((c / 16 * S_out + s) *
// kp / 32 + b) * 16 + c % 16, so a 32-segment unit of one input writes each
// group of 16 channels as one 2 KB stretch (the warp-specialised tensor-core
// F stage, the default where it applies; CELLSPE_FSTAGE_TC32=0 or 1, read per
// call, keeps layout 1).  A launch over a block of inputs writes at out +
// s0 * kp * 64 bytes; a block of channels c0 (a multiple of 16) onwards
// starts at c0 * S_out * kp * 4 bytes in both k-blocked layouts.
int cs_fstage_layout(const CsFStageArgs& a);
// Segment-major spectra [S][K][C] (tmp) -> the X stage's layout at out:
// F32 float2 rows (c, s), F16 half rows (c, plane, s); row pitch kp, S_out
// inputs per (c[, plane]) block (tmp and out already offset to the block).
int cs_spectra_transpose(const void* tmp, int S, int K, int C, int kp, int S_out, int format, void* out,
                         cudaStream_t st);
// fstage_tc.cu: the N = 2048 FP16-output F stage on the tensor cores (both
// DFT passes as tcgen05 MMAs).  cs_fx_fstage uses it for those arguments
// when the environment sets CELLSPE_FSTAGE_TC=1.
bool cs_fstage_tc_supported(const CsFStageArgs& a);
int cs_fx_fstage_tc(const CsFStageArgs& a, cudaStream_t st);
// Error code of the last tensor-core F-stage launch (0 = ok; 1, 2 = a wait
// timed out).  Call after the stream has synchronised.
int cs_fstage_tc_status(unsigned* code);
// fstage_tc32.cu: the N = 2048 tensor-core F stage with 32-segment units and
// k-blocked FP16 output (kblock = 1, K and kp multiples of 32), real-input
// symmetry halving the CUDA-core twiddle work; `specialised` selects the
// warp-specialised form.  cs_fx_fstage uses that form for those arguments
// unless CELLSPE_FSTAGE_TC32 is 0 (the warp FFT) or 1 (the lockstep form).
bool cs_fstage_tc32_supported(const CsFStageArgs& a);
int cs_fx_fstage_tc32(const CsFStageArgs& a, cudaStream_t st, bool specialised = false);
int cs_fstage_tc32_status(unsigned* code);

// xstage.cu -----------------------------------------------------------------
// FP32 CUDA-core X stage: spectra float2 [C][S][kp] (K used) -> vis float2
// [C][P], P = S(S+1)/2, p = i(i+1)/2 + j (j <= i), V = sum_k X_i conj(X_j).
int cs_xmac_f32(const float2* spectra, int S, int C, int K, int kp, float2* vis, int accumulate,
                cudaStream_t st);
// Tensor-core (tcgen05, FP16 in, FP32 accumulate) X stage:
// spectra __half [C][2][S][kp] (K used; kp % 8 == 0), or k-blocked
// [C][S][kp/32][2][32] with kblock = 1 (K, kp % 32 == 0), or channel-grouped
// k-blocked with kblock = 2 (C % 16 == 0; see cs_fstage_layout) -> vis
// float2 [C][P]; inv_scale [S*C] or null.
int cs_xmac_tc_f16(const void* spectra, int S, int C, int K, int kp, float2* vis, const float* inv_scale,
                   int scale_stride, int accumulate, cudaStream_t st,
                   int kblock = 0);   // inv_scale[s * scale_stride + c]
// INT8 X stage (legacy mma.sync IMMA: tcgen05 has no kind::i8 on sm_103a),
// int32 accumulate: planes int8 [C][2][S][kp] (K, kp % 32 == 0, K <= 65536),
// V_ij scaled by scale[i*stride + c] scale[j*stride + c].
int cs_xmac_i8(const int8_t* planes, int S, int C, int K, int kp, float2* vis, const float* scale, int scale_stride,
                  int accumulate, cudaStream_t st);
// FP32 spectra [C][S][kp] -> int8 planes [C][2][S][kp], per-row max-abs scale [S][C].
int cs_quantise_i8(const float2* spectra, int S, int C, int K, int kp, int8_t* planes, float* scale, cudaStream_t st);
// Error code of the last tensor-core X-stage launch (0 = ok; 1..3 = a
// pipeline wait timed out).  Call after the launching stream has synchronised.
int cs_xmac_tc_status(unsigned* code);
// Batched service jobs: job b's inputs are rows off .. off + S - 1 of a stacked
// job whose channel-major triangle is src [C][P_stacked]; its own triangle goes to
// dst ([C][P] or, baseline_major, [P][C]).
constexpr int CS_GATHER_MAX = 16;
struct CsGatherJob {
    int off, S;
    float2* dst;
    int baseline_major;
};
struct CsGatherArgs {
    int n, C;
    int64_t P_stacked;
    const float2* src;
    CsGatherJob job[CS_GATHER_MAX];
};
int cs_vis_gather(const CsGatherArgs& a, cudaStream_t st);
// Baseline-major <-> channel-major triangle transpose ([C][P] -> [P][C]).
int cs_vis_to_baseline_major(const float2* vis_cp, float2* vis_pc, int C, int64_t P, cudaStream_t st);

// spectrometer.cu -----------------------------------------------------------
struct CsSpecArgs {
    const uint8_t* planes;      // [nsub][bytes_per_sub] packed 2-bit, LSB first
    int64_t bytes_per_sub;
    int nsub;
    int N;                      // FFT points (1024 .. 65536)
    int overlap;
    int window;                 // 0 none, 1 cosine, 2 cosine^2
    int ffts_per_spectrum;      // K (non-overlapped)
    int nspec;
    float lut[4];
    float* power;               // [nsub][nspec][N/2+1]
    float* partial;             // scratch, cs_spectrometer_scratch_floats() floats
    // phase-cal (tonebins == 0 disables)
    int tonebins, rotatorlen, ntones;
    double pcal_offset_hz, fs_hz;
    float2* pcal_bins;          // [nsub][nspec][tonebins]
    float2* pcal_tones;         // [nsub][nspec][ntones] or null
    // Optional caller-owned tables (null: the cached tables of this library)
    const float2* tw_table;     // exp(-2 pi i m / N), N entries
    const float* win_table;     // window, N entries
    const float2* rot_table;    // pcal rotator, rotatorlen entries
    int ffts_per_chunk;         // FFTs per partial spectrum (0: default)
    const uint32_t* valid_mask; // bit t: sample time t of the planes is data (null: all data)
    int pcal_sources;           // sources sharing the call's FFT count (0 or 1: one)
    int pcal_source;            // this source's index among them
    int skip_power;             // 1: phase-cal only (no power spectra)
};
int64_t cs_spectrometer_scratch_floats(const CsSpecArgs& a);
int64_t cs_spectrometer_pcal_floats(const CsSpecArgs& a);   // the phase-cal part of it
int cs_spectrometer(const CsSpecArgs& a, cudaStream_t st);
// Window function of TaskCoreIPP::generate_windowfunction, n floats (cached).
const float* cs_window_table(int type, int n);

// spectrometer_xpol.cu: two sources and their cross spectrum.
// Overlapped, windowed windows of one 2-bit plane (LSB first, optional
// validity mask): out[nspec * novl][N] floats, window j of spectrum s from
// sample s*K*N + j*N/overlap.
int cs_spec_windows(const uint8_t* plane, const uint32_t* vmask, int N, int overlap, int K, int nspec, int window,
                    const float lut[4], float* out, cudaStream_t st);
// X0, X1: [nspec * novl][N/2+1] spectra -> power [2][nspec][N/2+1] (autos of
// both sources) and xpol [nspec][N/2+1] (X0 conj X1, DC / Nyquist real).
int cs_xpol_reduce(const float2* X0, const float2* X1, int N, int overlap, int K, int nspec, float* power,
                   float2* xpol, cudaStream_t st);

// framed.cu (framed Mark5B and VDIF input) --------------------------------
// Geometry of a framed stream: frame f starts at offset + f * frame_bytes
// (offset on the device for Mark5B, 0 for VDIF), its payload at
// payload_offset bytes into the frame (frame0_payload_offset for frame 0).
struct CsFraming {
    int64_t frame_bytes;
    int payload_bytes;
    int payload_offset;
    int frame0_payload_offset;
    int nch;                      // 2-bit channels per sample time: 1, 2, 4, 8, 16
};
// VDIF header-time check (mark5_format_vdif_validate): frames whose number is
// a multiple of `granularity` must carry the time predicted from frame 0.
struct CsVdifClock {
    CsFraming fmt;
    double frame_ns;              // payload bits * 1000 / Mbps
    long long step_ns;            // gframens / granularity (integer division)
    int granularity;
    int mjd0, sec0, ns0;          // time of frame 0
    int epoch_mjd[64];            // MJD of each VDIF reference epoch
};
// Frame search + per-frame valid byte ranges (fill-pattern blanking); the
// offset of the first frame stays on the device (no frame found: >= 1 MiB).
int cs_m5b_locate(const uint8_t* framed, int64_t bytes, int* d_offset, int2* ranges, int64_t nframes, cudaStream_t st);
// VDIF validity per frame (all or nothing): header time, invalid bit and
// fill pattern; blanked frames counted into *d_blanked (cleared first).
int cs_vdif_locate(const uint8_t* framed, int64_t bytes, const CsVdifClock& clk, int2* ranges, int64_t nframes,
                   unsigned long long* d_blanked, cudaStream_t st);
// mark5_stream_decode: nsamp samples per channel into nch float planes,
// unblanked count added to *d_good (cleared first).  d_offset null = 0.
int cs_framed_decode(const uint8_t* framed, int64_t bytes, const CsFraming& fmt, const int* d_offset,
                     const int2* ranges, int64_t nsamp, const float lut[4], float* out, unsigned long long* d_good,
                     cudaStream_t st);
// Payload bytes back to back (nframes * payload_bytes) and, if mask != null,
// one validity bit per sample time.
int cs_framed_deframe(const uint8_t* framed, int64_t bytes, const CsFraming& fmt, const int* d_offset,
                      const int2* ranges, int64_t nframes, uint8_t* payload, uint32_t* mask, cudaStream_t st);
// Per-channel 2-bit planes ([nch][ngroups] words of 16 samples) plus the
// validity mask (ceil(ngroups/2) words), straight from the framed bytes.
int cs_framed_planes(const uint8_t* framed, int64_t bytes, const CsFraming& fmt, const int* d_offset,
                     const int2* ranges, int64_t nframes, int64_t ngroups, uint32_t* planes, uint32_t* mask,
                     cudaStream_t st);

// dsp.cu (task-API vector primitives) ---------------------------------------
int cs_cmac(const float2* a, const float2* b, float2* acc, int64_t n, int conj_b, cudaStream_t st);
int cs_cmul(const float2* a, const float2* b, float2* out, int64_t n, cudaStream_t st);
int cs_cadd(const float2* a, const float2* b, float2* out, int64_t n, cudaStream_t st);
int cs_sincos(const float* arg, float2* cossin, int64_t n, int normalized, cudaStream_t st);
int cs_sincos_generator(float start, float inc, float2* cossin, int64_t n, cudaStream_t st);
int cs_autocorr_acc(const float2* x, float2* acc, int64_t n, cudaStream_t st);
int cs_reciprocal(const float* in, float* out, int64_t n, cudaStream_t st);
int cs_fadd(const float* x, float* acc, int64_t n, cudaStream_t st);      // acc += x

// runtime.cpp: checks shared by entry points defined in other files ---------
// The four levels that `format` (CELLSPE_LEVELS_*) or `custom` names; false
// for an unknown table.
bool cs_pick_levels(int format, const float* custom, float out[4]);
// The argument checks every spectrometer entry point runs; 0 or a
// CELLSPE_ERR_* code with the error text set ("who" names the caller).
int cs_spec_check(const cellspe_spec_params* p, const char* who);
