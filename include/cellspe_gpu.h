/*
 * cellspe_gpu.h -- GB300 FX correlator / spectrometer engine, C ABI.
 *
 * Direct entry points for the hot path behind the task API.  Every function
 * takes plain pointers and sizes, returns 0 on success or a CELLSPE_ERR_*
 * code, and blocks until its results are in the caller's output buffers.
 * `memory` says where the buffers live: CELLSPE_MEM_HOST (the engine copies
 * inputs to the GPU and results back; pinned memory from cellspe_host_alloc
 * is fastest) or CELLSPE_MEM_DEVICE (device pointers on the engine's GPU).
 * Calls from several host threads are safe; each thread uses its own stream
 * and workspace.  A call's first kernel waits (on the device) for all work
 * issued before the call to the legacy default stream, so device buffers
 * filled there, or on blocking streams, are ready; work on the caller's own
 * non-blocking streams must be synchronised by the caller.  There is no CPU
 * fallback: without a usable GPU every call fails with CELLSPE_ERR_CUDA and
 * cellspe_last_error() says why.
 */
#ifndef CELLSPE_GPU_H
#define CELLSPE_GPU_H

#include "cellspe-tasklib.h"

#ifdef __cplusplus
extern "C" {
#endif

#define CELLSPE_MEM_HOST    0
#define CELLSPE_MEM_DEVICE  1

#define CELLSPE_OK               0
#define CELLSPE_ERR_ARG          1   /* invalid argument                  */
#define CELLSPE_ERR_UNSUPPORTED  2   /* size or mode not implemented      */
#define CELLSPE_ERR_NOMEM        3   /* job exceeds the HBM budget         */
#define CELLSPE_ERR_CUDA         4   /* CUDA runtime error                 */
#define CELLSPE_ERR_INJECTED     5   /* failure injected by the test hook  */

/* 2-bit level tables (value = levels[bit0 + 2*bit1]). */
#define CELLSPE_LEVELS_MARK5B        0  /* {-3.3359, +1, -1, +3.3359}  mark5_format_mark5b.c:63  */
#define CELLSPE_LEVELS_TWOBIT        1  /* {+1, -1, +3.3359, -3.3359}  DataUnpackers.cpp:195     */
#define CELLSPE_LEVELS_OFFSET_BINARY 2  /* {-3.336, -1, +1, +3.336}    synthetic offset binary    */
#define CELLSPE_LEVELS_VDIF          3  /* {-3.3359, -1, +1, +3.3359}  format_vdif.c:70          */
#define CELLSPE_UNPACK_MSB_FIRST     0x100  /* single channel: sample 0 in bits 7:6 */

/* X-stage arithmetic */
#define CELLSPE_X_FP32     0   /* FP32 CUDA cores                                   */
#define CELLSPE_X_TC_FP16  1   /* tcgen05 tensor cores, FP16 inputs, FP32 accumulate */
#define CELLSPE_X_INT8     2   /* int8 spectra (per input and channel max-abs scale),
                                  mma.sync IMMA, int32 accumulate; K % 16 == 0.
                                  tcgen05 has no kind::i8 on sm_103a */

/* Visibility layout */
#define CELLSPE_VIS_CHANNEL_MAJOR   0  /* vis[C][P]  (X-engine order)            */
#define CELLSPE_VIS_BASELINE_MAJOR  1  /* vis[P][C]  (one spectrum per product)   */

/* ---- engine control ---------------------------------------------------- */
const char* cellspe_last_error(void);          /* this thread's last error text */
int  cellspe_device_count(void);
int  cellspe_set_hbm_budget(long long bytes);  /* admission limit per job (0 = 90% of free) */
long long cellspe_get_hbm_budget(void);
void* cellspe_host_alloc(size_t bytes);        /* pinned host memory */
void cellspe_host_free(void* p);
void* cellspe_device_alloc(size_t bytes);
void cellspe_device_free(void* p);
int  cellspe_memcpy(void* dst, const void* src, size_t bytes, int kind); /* 1 H2D, 2 D2H, 3 D2D */
/* Fault injection for tests: the next `count` tasks or calls on `slot`
 * (-1 = direct calls) fail with CELLSPE_ERR_INJECTED before touching the GPU. */
int  cellspe_debug_inject_failure(int slot, int count);
/* Kernels this library has launched since it was loaded (all threads). */
long long cellspe_kernel_launches(void);
/* Device time in ms of the calling thread's last blocking FX job, measured
 * with CUDA events on the engine stream: [0] delay model, [1] F stage
 * (unpack + FFT + phasor), [2] X stage, [3] output layout/copies. */
int  cellspe_last_stage_times(float* ms, int n);

/* ---- K-a: 2-bit unpack ----------------------------------------------------
 * out: nchan planes of nsamp floats.  Bit-exact with the reference decode
 * (mark5_format_mark5b.c:1852-1915, DataUnpackers.cpp:174-288). */
int cellspe_unpack2bit(const void* raw, long long nsamp, int nchan, int format,
                       const float* custom_levels, float* out, int memory);

/* ---- K-b: FFTs ------------------------------------------------------------
 * Forward, unscaled.  C2C: interleaved complex, n in [16, 16384], replaces
 * _fft_1d_r2 / exec_FFT (cellspe-tasklib-dsp.cpp:565-602).  R2C: n reals ->
 * n/2+1 bins, n in [32, 32768], replaces genericFFTexec_R (architecture.h:563). */
int cellspe_fft_c2c(const void* in, void* out, int n, long long batch, int memory);
int cellspe_fft_r2c(const float* in, void* out, int n, long long batch, int memory);
/* R2C with IPP "Perm" packing, the layout ippsDFTFwd_RToPerm_32f writes and
 * TaskCoreIPP::doMaths reads (spectrometer/src/IA-32/TaskCoreIPP.cpp:116, 430,
 * 438-439): n floats per row, [R0, R_{n/2}, Re X1, Im X1, ..., Re X_{n/2-1},
 * Im X_{n/2-1}]; forward, unscaled; n a power of two in [32, 32768]. */
int cellspe_fft_r2c_perm(const float* in, float* out, int n, long long batch, int memory);

/* ---- XF lag products -------------------------------------------------------
 * lags[p][m] = scale * sum_c vis[p][c] exp(+2 pi i c m / C): the backward,
 * unnormalised transform of each product's visibility spectrum, as zerocorr's
 * FFTW_BACKWARD plan (mark5access examples/zerocorr.c:391, 626-645; lag j is
 * element j for j >= 0 and j + C for j < 0; scale = 1/#FFTs there).
 * vis, lags: complex64 [P][C] (baseline-major), C a power of two <= 16384. */
int cellspe_vis_lags(const void* vis, void* lags, long long n_products, int n_channels, double scale, int memory);

/* ---- Spectrum accumulation ---------------------------------------------------
 * acc[i] += add[i] for n floats on the GPU: the ippsAdd_32f_I / ippsAdd_32fc_I
 * summation of TaskCoreIPP::combineResults (spectrometer/src/IA-32/
 * TaskCoreIPP.cpp:311-349), used by the TaskCoreCUDA plug-in to add a core's
 * sub-spectra into the dispatcher's common spectra.  Both pointers in the
 * memory space `memory` names. */
int cellspe_accumulate_f32(float* acc, const float* add, long long n, int memory);

/* ---- K-d: X stage on precomputed spectra ----------------------------------
 * spectra complex64 [C][S][K] (FP32 mode) -> vis complex64 [C][P] (channel-major),
 * V_ij = sum_k X_i conj(X_j), j <= i, p = i(i+1)/2 + j.
 * Replaces genericAddProduct_32fc_conj (architecture.h:427-433) looped over
 * products, three_baseline_naive_MACauto (minicorrelator_spu.c:745-786). */
int cellspe_xmac(const void* spectra, int S, int C, int K, void* vis, int accumulate, int memory);
/* Tensor-core X stage on FP16 spectra, layout half [C][2][S][K] (plane 0 Re,
 * plane 1 Im, K a multiple of 8) -> vis complex64 [C][P], FP32 accumulation. */
int cellspe_xmac_f16(const void* spectra_f16, int S, int C, int K, void* vis, int accumulate, int memory);
/* INT8 X stage: int8 spectra planes [C][2][S][K] (plane 0 Re, plane 1 Im,
 * K a multiple of 16, at most 65536) with a dequantisation scale [S][C] ->
 * vis complex64 [C][P], V_ij = scale[i][c] scale[j][c] sum_k q_i conj(q_j),
 * the integer sums exact (int32) and scaled in FP32.  Warp-level mma.sync
 * IMMA: tcgen05 has no kind::i8 on sm_103a. */
int cellspe_xmac_i8(const void* planes_i8, const float* scale, int S, int C, int K, void* vis, int accumulate,
                    int memory);
/* Parameters of CELLDSP_TASK_XMAC (input vector 0). */
typedef struct { int S, C, K, accumulate; } cellspe_xmac_params;

/* ---- Full FX correlation: unpack -> FFT -> delay/fringe -> X --------------- */
typedef struct {
    int    n_inputs;          /* S: stations x polarisations                       */
    int    fft_points;        /* N: 512 .. 32768, power of two; C = N/2 channels   */
    int    n_segments;        /* K: FFT segments integrated                        */
    int    x_mode;            /* CELLSPE_X_*                                        */
    int    vis_order;         /* CELLSPE_VIS_*                                      */
    int    levels;            /* CELLSPE_LEVELS_* (| CELLSPE_UNPACK_MSB_FIRST)      */
    long long bytes_per_input;/* raw bytes per input (multiple of 16)              */
    long long start_sample;   /* sample index of segment 0 inside each input        */
    double sample_rate_hz;    /* fs (delay model)                                   */
    double lo_freq_hz;        /* sky frequency of channel 0 (fringe rotation)       */
    int    accumulate;        /* 1: vis += result, 0: vis = result                  */
    int    memory;            /* CELLSPE_MEM_*                                      */
    const float* custom_levels;   /* 4 floats overriding `levels`, or NULL          */
    const float* channel_scale;   /* [S][C] F-stage scale for the FP16 path, or NULL */
} cellspe_fx_params;

/* raw: S inputs of bytes_per_input bytes, 2-bit single channel, 4 samples per
 * byte.  delay_poly: [S][4] seconds, tau(t) = sum_m poly[m] t^m with t the
 * segment centre in seconds from start_sample, or NULL for no delay model.
 * Segment k of input s starts at start_sample + k*N + round(tau*fs); its
 * spectrum is multiplied by exp(i*(2 pi lo tau + 2 pi c (fs/N) tau_frac)).
 * vis: C*P complex64 in vis_order. */
int cellspe_fx_correlate(const cellspe_fx_params* p, const void* raw, const double* delay_poly, void* vis);
/* Device bytes the engine needs for this job (admission control). */
long long cellspe_fx_workspace_bytes(const cellspe_fx_params* p);
/* Asynchronous form on a caller's CUDA stream (cudaStream_t passed as void*).
 * Device memory only; the workspace stays owned by the calling thread until
 * cellspe_release_workspace().  Captures into CUDA graphs once the workspace
 * has been sized by one earlier call. */
int cellspe_fx_correlate_async(const cellspe_fx_params* p, const void* raw, const double* delay_poly,
                               void* vis, void* stream);
int cellspe_release_workspace(void);

/* ---- Correlation service: continuous batching ----------------------------
 * Jobs (cellspe_fx_params + buffers) are queued on submit and return at once.
 * max_streams worker threads, each with its own CUDA stream and device
 * workspace, take the oldest queued job as soon as its device footprint
 * (cellspe_fx_workspace_bytes) fits next to the jobs already running under
 * hbm_budget_bytes, so jobs that arrive while others run are admitted as
 * memory frees and their work overlaps on the GPU.  Results are identical to
 * cellspe_fx_correlate on the same job (same kernels, deterministic order).
 * Jobs of fewer than priority_samples samples (inputs x points x segments)
 * run on a high-priority stream, so the GPU schedules their thread blocks
 * ahead of the waiting blocks of larger jobs' kernels.  With large_samples > 0,
 * jobs of at least that many samples run one at a time: a queued large job
 * waits while another large job runs, and the jobs queued behind it are
 * admitted past it (off by default: on the serving mix it did not lower the
 * p99 latency).  Each large kernel fills the GPU on its own, so jobs that run
 * side by side all finish late: two streams keep the p99 latency near the
 * largest job's own run time while small jobs pass large ones.  Workers use the F-stage schedule that a direct call has timed (they
 * time none themselves).  Unless batch_inputs < 0, a worker that takes a small
 * job (device buffers, at most 16 inputs, tensor-core X stage, no delay
 * model, scale, custom levels or accumulation) also takes the queued jobs of
 * the same shape (FFT size, segments, input length, start sample, levels)
 * up to batch_inputs inputs in all, and runs them as one stacked job: one
 * F-stage and one X-stage launch, each job's triangle then gathered into its
 * own visibility buffer (the values equal each job's solo run).
 * Buffers must stay valid until cellspe_service_wait returns for the job. */
typedef struct cellspe_service cellspe_service;
typedef struct {
    long long hbm_budget_bytes;   /* 0: 80% of free device memory            */
    int       max_streams;        /* concurrent jobs (0: 2)                    */
    int       batch_inputs;       /* small jobs batched up to this many inputs (<= 128); 0: 64; < 0: off */
    long long priority_samples;   /* 0: 2^24; < 0: one priority for all jobs */
    long long large_samples;      /* <= 0: no limit (large jobs may overlap)  */
} cellspe_service_config;
typedef struct {
    long long completed, failed, queued;
    int       running, max_running;
    double    p50_ms, p99_ms;     /* submit -> done latency of completed jobs */
    double    p99_queue_ms;       /* submit -> start                          */
    long long budget_bytes;
    long long batched_jobs;       /* jobs that ran in a shared launch          */
    long long batched_launches;   /* stacked jobs those formed                 */
} cellspe_service_stats;
cellspe_service* cellspe_service_create(const cellspe_service_config* cfg);
int  cellspe_service_submit(cellspe_service* s, const cellspe_fx_params* p, const void* raw,
                            const double* delay_poly, void* vis, long long* job_id);
int  cellspe_service_wait(cellspe_service* s, long long job_id, double* latency_ms);
int  cellspe_service_get_stats(cellspe_service* s, cellspe_service_stats* out);
void cellspe_service_destroy(cellspe_service* s);

/* ---- Spectrometer ----------------------------------------------------------
 * Restates TaskCoreIPP::doMaths (TaskCoreIPP.cpp:394-513) on the GPU for every
 * subband of a 2-bit stream. */
#define CELLSPE_SPEC_INTERLEAVED 0  /* raw: nsub channels interleaved per sample time (Mark5B payload) */
#define CELLSPE_SPEC_PLANES      1  /* raw: nsub planes of bytes_per_sub bytes, 1 channel each */
#define CELLSPE_SPEC_MARK5B_FRAMED 2 /* raw: a framed Mark5B recording (16-byte headers, 10000-byte
                                      * payloads, n_subbands = 4, 8 or 16 channels); headers are
                                      * stripped and fill-pattern zones blanked (decoded as 0.0)
                                      * on the device, as cellspe_mark5b_decode does; samples past
                                      * the last complete frame are blanked too */
#define CELLSPE_SPEC_VDIF_FRAMED   3 /* raw: a framed VDIF recording from byte 0 (n_subbands = 1, 4, 8
                                      * or 16 channels, 2-bit, frames of at least 528 bytes); frames
                                      * are validated and blanked as cellspe_vdif_decode does, with
                                      * Mbps = sample_rate_hz * 2 * n_subbands / 1e6 (a whole number);
                                      * levels should be CELLSPE_LEVELS_VDIF */
typedef struct {
    int    fft_points;        /* N: 1024 .. 65536                                  */
    int    overlap;           /* fft_overlap_factor                                */
    int    window;            /* WindowFunctionType: 0 none, 1 cosine, 2 cosine^2,
                               * 3 Hamming, 4 Hann, 5 Blackman (alpha 0.5)          */
    int    ffts_per_spectrum; /* K non-overlapped FFTs per spectrum                 */
    int    n_spectra;
    int    n_subbands;        /* 1, 4, 8 or 16                                      */
    int    input_layout;      /* CELLSPE_SPEC_*                                     */
    int    levels;            /* CELLSPE_LEVELS_*                                   */
    long long raw_bytes;      /* total raw bytes                                    */
    int    pcal_tonebins;     /* 0 disables phase-cal                               */
    int    pcal_rotatorlen;
    int    pcal_ntones;
    double pcal_offset_hz;
    double sample_rate_hz;
    int    memory;
    const float* custom_levels;
} cellspe_spec_params;

/* power: [nsub][nspec][N/2+1] float; pcal_bins: [nsub][nspec][tonebins]
 * complex64 (may be NULL when pcal is off); pcal_tones: [nsub][nspec][ntones]
 * complex64 or NULL. */
int cellspe_spectrometer(const cellspe_spec_params* p, const void* raw, float* power,
                         void* pcal_bins, void* pcal_tones);
long long cellspe_spectrometer_workspace_bytes(const cellspe_spec_params* p);

/* Two recordings (sources) and their cross-polarisation spectrum:
 * TaskCoreIPP::doMaths with two sources and one cross product
 * (spectrometer/src/IA-32/TaskCoreIPP.cpp:394-513).  raw0 and raw1 are two
 * recordings in the layout p describes (p->raw_bytes each, p->n_subbands
 * channels); channel0 / channel1 pick the subband of each (UseFile1Channel - 1,
 * UseFile2Channel - 1).  Outputs, n = p->n_spectra, nb = fft_points/2 + 1:
 *   power     [2][n][nb] float     auto spectra of source 0 and source 1
 *   xpol      [n][nb] complex64    sum X0 conj(X1) over the overlapped FFTs;
 *                                  bins 0 and nb-1 real (Re X0 Re X1)
 *   pcal_bins [2][n][tonebins] complex64 or NULL; as in the reference the FFT
 *             count advances after each source's FFT, so with overlap 2 source
 *             0 folds every overlapped window and source 1 none.
 * All spectra are scaled by 1/(overlap*K - (overlap-1)).  fft_points up to
 * 32768. */
int cellspe_spectrometer_xpol(const cellspe_spec_params* p, const void* raw0, const void* raw1, int channel0,
                              int channel1, float* power, void* xpol, void* pcal_bins);

/* ---- framed Mark5B input ------------------------------------------------
 * A Mark5B recording is a run of 10016-byte frames: a 16-byte header (sync
 * word 0xABADDEED, frame number, BCD time code) and 10000 bytes of 2-bit
 * samples, nchan channels interleaved per sample time (mark5access
 * mark5_format_mark5b.c).  Missing data carry the fill pattern 0x11223344
 * and are blanked per payload by the rules of blanker_mark5.c. */
typedef struct {
    long long first_frame_offset;  /* byte offset of the first frame (-1: none)        */
    long long frames;              /* complete frames from there to the buffer end    */
    long long good_samples;        /* cellspe_mark5b_decode: unblanked samples per
                                    * channel, or -1 when the frames ran out (the
                                    * value mark5_stream_decode returns)              */
    int mjd;                       /* 56000 + BCD day digits of the first header, as
                                    * FileSource::locateFirstHeader reads them        */
    int seconds;                   /* BCD seconds of day of the first header          */
    int frame_number;              /* 15-bit frame number within the second           */
    int reserved;
} cellspe_mark5b_info;

/* new_mark5_stream_memory(framed, bytes) + mark5_stream_decode(nsamp):
 * finds the first frame (sync word twice, 10016 bytes apart, within the first
 * MiB; mark5_format_mark5b.c:98-131), strips the headers and decodes nsamp
 * samples of each of nchan (4, 8, 16) channels into out[nchan][nsamp] with the
 * mark5access levels {-3.3359, +1, -1, +3.3359}; blanked samples are 0.0.
 * Like the library, it stops writing after the last complete frame and then
 * reports good_samples = -1 (also when the last wanted sample ends the last
 * frame).  Returns CELLSPE_ERR_ARG when no frame is found.  info may be NULL.
 * memory = CELLSPE_MEM_HOST or _DEVICE for framed and out. */
int cellspe_mark5b_decode(const void* framed, long long bytes, int nchan, long long nsamp, float* out,
                          int memory, cellspe_mark5b_info* info);

/* FileSource::read for framed data (spectrometer/src/FileSource.cpp:185-215):
 * the payloads of `frames` frames from the first frame on, back to back,
 * into payload[frames * 10000]; with valid_mask != NULL also one bit per
 * sample time (bit t % 32 of word t / 32 set = unblanked), nchan channels per
 * sample time.  frames = 0 takes every complete frame; payload and the mask
 * must hold that many (see info->frames, filled first).  info may be NULL. */
int cellspe_mark5b_deframe(const void* framed, long long bytes, int nchan, long long frames, void* payload,
                           unsigned int* valid_mask, int memory, cellspe_mark5b_info* info);

/* ---- framed VDIF input ---------------------------------------------------
 * A VDIF recording is a run of frames from byte 0, each a 32-byte header (16
 * with the legacy bit, word 0 bit 30) and a payload of 2-bit samples, nchan
 * channels interleaved per sample time, channel c in bits 2c..2c+1 of the
 * sample time's bit field (mark5access format_vdif.c).  The frame length is
 * word 2 of the first header.  The decode restates a mark5access memory
 * stream opened with the format "VDIF_<payload>-<mbps>-<nchan>-2"
 * (new_mark5_stream_memory + mark5_stream_decode):
 *   - a frame is used whole or blanked whole (decoded as 0.0);
 *   - frames after the first are blanked when the invalid bit (word 0 bit 31)
 *     is set, or when, on frame numbers that are multiples of the frame-time
 *     granularity, the header time (reference epoch + seconds + frame number
 *     x frame duration) differs from the time predicted from the first frame
 *     (mark5_format_vdif_validate, format_vdif.c:2299-2337; frame duration
 *     payload * 8000 / mbps ns; its integer-ns granularity and the integer
 *     step per frame as the library computes them);
 *   - any frame is blanked when the first or last 64-bit word of its payload
 *     is the fill pattern 0x1122334411223344 (blanker_vdif);
 *   - like the library, frame 0 of a legacy stream is read from byte 32 of
 *     the frame (the library sets the first payload pointer before it learns
 *     the header is 16 bytes, format_vdif.c:2196-2220).
 * At least two frames are required. */
typedef struct {
    long long frames;          /* complete frames in the buffer                     */
    long long good_samples;    /* cellspe_vdif_decode: unblanked samples per channel,
                                * or -1 when the frames ran out (the value
                                * mark5_stream_decode returns)                      */
    long long blanked_frames;  /* frames of the buffer that are blanked             */
    int frame_bytes;           /* header + payload, from the first header           */
    int header_bytes;          /* 32, or 16 with the legacy bit                     */
    int mjd, seconds, ns;      /* time of the first frame (ns rounded)              */
    int frame_number;          /* of the first frame, within its second             */
    int nchan_header;          /* 2^(word 2 bits 24..28)                            */
    int thread_id, station_id;
    int reserved;
} cellspe_vdif_info;

/* Decodes nsamp samples of each of nchan (1, 2, 4, 8, 16) channels into
 * out[nchan][nsamp] with the VDIF levels {-3.3359, -1, +1, +3.3359}; nsamp a
 * multiple of 4 / nchan for nchan < 4.  Like the library, it stops writing
 * after the last complete frame and then reports good_samples = -1 (also when
 * the last wanted sample ends the last frame).  mbps: the stream's total bit
 * rate in Mbit/s.  memory = CELLSPE_MEM_HOST or _DEVICE for framed and out;
 * info may be NULL. */
int cellspe_vdif_decode(const void* framed, long long bytes, int nchan, int mbps, long long nsamp, float* out,
                        int memory, cellspe_vdif_info* info);

/* The payloads the decoder reads, of `frames` frames (0 = every complete
 * frame), back to back into payload[frames * payload bytes]; with
 * valid_mask != NULL also one bit per sample time (bit t % 32 of word t / 32
 * set = used).  info is filled first (frames, frame_bytes, header_bytes). */
int cellspe_vdif_deframe(const void* framed, long long bytes, int nchan, int mbps, long long frames, void* payload,
                         unsigned int* valid_mask, int memory, cellspe_vdif_info* info);

/* Spectrometer that allocates no device memory (no counterpart in the
 * reference).  For callers that cannot call cudaMalloc when they run it:
 * real-time loops that must not stall on the allocator (cudaMalloc/cudaFree
 * can synchronise the device), code running during CUDA graph capture, or
 * hosts that fix the library's device footprint up front.  Same results as
 * cellspe_spectrometer (within FP32 summation order), enqueued on `stream`
 * (a cudaStream_t, NULL = default stream) without synchronising.
 * Requirements: memory = CELLSPE_MEM_DEVICE (raw, power, pcal_* are device
 * pointers); input_layout = CELLSPE_SPEC_PLANES unless n_subbands == 1 (never framed);
 * fft_points <= 65536; pcal_rotatorlen <= 65536.
 * Scratch: a fixed static device array of 4,194,304 floats (16 MiB) plus
 * 1.25 MiB of tables, held by every GPU that loads the library until exit.
 * Jobs whose partial spectra do not fit are rejected with CELLSPE_ERR_ARG.
 * The first call on each device looks up the arrays' device addresses
 * (cudaGetSymbolAddress): make it before any stream capture.  All calls
 * share the arrays: calls that overlap on the GPU race. */
int cellspe_spectrometer_noalloc(const cellspe_spec_params* p, const void* raw, float* power,
                                 void* pcal_bins, void* pcal_tones, void* stream);

#ifdef __cplusplus
}  /* extern "C" */
#endif

#endif /* CELLSPE_GPU_H */
