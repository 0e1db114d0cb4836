/* CPU oracle for the GB300 FX correlator / spectrometer hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the
 * reference's CPU semantics for the hot path; it exists to check the CUDA
 * path and to time the CPU baseline.  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg may load it.  The product library never
 * links or calls it, and there is no CPU fallback in the product.
 *
 * Parity pins (checked by tests/test_oracle_golden.py):
 *   - orc_unpack2bit with the Mark5B table is compared bit-for-bit with the
 *     reference's mark5access 1.4.3 decode (compiled from the reference tree
 *     into oracle/_ref/libref_mark5.so) and with committed golden vectors.
 *   - orc_addproduct_32fc(_conj) are compared bit-for-bit with the reference's
 *     GENERIC kernels of architecture.h (oracle/_ref/libref_generic.so).
 *   - The FFT has no reference pin: FFTW / IPP / the Cell SDK FFT are not
 *     available (parity unpinned for the FFT); it is checked against an
 *     FP64 DFT and against analytic known answers.
 *   - The PCal fold follows TaskCoreIPP::extract_PCal and is checked with the
 *     reference's own PCal unit-test recipe (tone phases within 0.1 deg).
 */
#ifndef CELLSPE_ORACLE_H
#define CELLSPE_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct { float re, im; } orc_cf32;

/* 2-bit multi-channel unpack.  nchan channels are interleaved per sample
 * time, 2 bits each, so one sample time spans nchan/4 bytes (nchan>=4) or a
 * quarter byte (nchan==1).  Field (t, c) starts at bit 2*(t*nchan + c) of the
 * little-endian byte stream when msb_first==0 (mark5access Mark5B and
 * cellspe TwoBitUnpacker order), or, when msb_first==1 (single channel only),
 * sample 0 sits in bits 7:6 of byte 0 (TwoBitSinglechannelUnpacker order).
 * code = bit0 + 2*bit1 of the field; value = lut[code].
 * out: nchan planes of nsamp floats, channel-major.
 * Restates mark5_format_mark5b.c:59-95 (initluts) + :1852-1915 and
 * spectrometer/src/IA-32/DataUnpackers.cpp:174-227, :244-288. */
void orc_unpack2bit(const uint8_t* raw, int64_t nsamp, int nchan, int msb_first,
                    const float lut[4], float* out);

/* Framed Mark5B (10016-byte frames: 16-byte header + 10000-byte payload).
 * orc_mark5b_find_first_frame restates findfirstframe
 * (mark5_format_mark5b.c:98-131): the first offset where the sync word
 * 0xABADDEED appears twice, 10016 bytes apart, searching at most 1 MiB.
 * orc_mark5b_valid_range restates blanker_mark5 (blanker_mark5.c) for one
 * 10000-byte payload (a single 32 KiB blanking zone): the byte range
 * [start, end) outside of which samples are blanked (decoded as 0).
 * orc_mark5b_decode_framed restates mark5_stream_decode on a memory stream:
 * nsamp samples per channel from the first frame on, lut2bit values inside
 * the valid range, 0.0 outside.  nchan = 4, 8 or 16 (2-bit).  Returns the
 * number of unblanked samples, or -1 when the frames run out (the decoder
 * steps to the next frame as soon as a payload is used up, so -1 also when
 * the last wanted sample ends the last frame), or when no frame is found. */
int orc_mark5b_find_first_frame(const uint8_t* data, int64_t bytes);
void orc_mark5b_valid_range(const uint8_t* payload, int* start, int* end);
int64_t orc_mark5b_decode_framed(const uint8_t* framed, int64_t bytes, int nchan, int64_t nsamp, float* out);

/* Framed VDIF, 2-bit real samples, as a mark5access memory stream opened with
 * the format "VDIF_<databytes>-<mbps>-<nchan>-2" (format_vdif.c 1.4.3).
 * The first frame starts at byte 0; word 2 of its header gives the frame
 * length (8-byte units) and the legacy bit (word 0 bit 30) a 16-byte instead
 * of a 32-byte header (mark5_format_vdif_init, format_vdif.c:2121-2257).
 * orc_vdif_frame_ok restates, for frame f >= 1, mark5_format_vdif_validate
 * (format_vdif.c:2299-2337: header time against the time predicted from the
 * first frame on frames f % framegranularity == 0, then the invalid bit) and
 * for every frame blanker_vdif (blanker_mark5.c:282-316: fill pattern in the
 * first or the last 64-bit payload word blanks the frame); frame 0 is not
 * validated (mark5_stream_next_frame, mark5_stream.c:144-193, runs only on
 * the frames after it).  orc_vdif_decode_framed decodes nsamp samples per
 * channel (nchan = 1, 2, 4, 8, 16) with the VDIF levels {-H, -1, +1, +H};
 * returns the unblanked sample count, -1 when the frames run out (also when
 * the last wanted sample ends the last frame), -2 on a header it cannot use
 * or a buffer shorter than two frames, -3 when nsamp is not a multiple of the
 * samples per byte.  Frame 0 of a legacy (16-byte header) stream is read from
 * byte 32, as the library does when the format name is "VDIF_...". */
int orc_vdif_frame_ok(const uint8_t* framed, int64_t bytes, int mbps, int64_t f);
/* time of frame 0 as the stream reads it (ms->mjd, ms->sec, ms->ns) */
int orc_vdif_first_time(const uint8_t* framed, int64_t bytes, int mbps, int* mjd, int* sec, int* ns);
int64_t orc_vdif_decode_framed(const uint8_t* framed, int64_t bytes, int nchan, int mbps, int64_t nsamp, float* out);

/* acc[i] += a[i]*b[i]            architecture.h:405-421 (do_complex_mac)  */
void orc_addproduct_32fc(const orc_cf32* a, const orc_cf32* b, orc_cf32* acc, int n);
/* acc[i] += a[i]*conj(b[i])      architecture.h:427-433                   */
void orc_addproduct_32fc_conj(const orc_cf32* a, const orc_cf32* b, orc_cf32* acc, int n);

/* Forward complex FFT, unscaled, e^{-2 pi i k n / N}, N a power of two.
 * Radix-2 DIT with FP64-computed twiddles.  The same transform as
 * fft_1d_r2_modified.h (_fft_1d_r2), exec_FFT and FFTW's forward C2C. */
void orc_cfft_f32(const orc_cf32* in, orc_cf32* out, int n);
void orc_cfft_f64(const double* in_reim, double* out_reim, int n);

/* Real-input forward FFT, N points -> N/2+1 bins (FFTW r2c layout; bins 0
 * and N/2 have zero imaginary part).  FP32 arithmetic through an N/2-point
 * complex FFT and the standard split post-processing. */
void orc_rfft_f32(const float* in, orc_cf32* out, int n);

/* Spectrometer, one source.  Restates TaskCoreIPP::doMaths
 * (spectrometer/src/IA-32/TaskCoreIPP.cpp:394-513) for one input:
 * overlapped windowed real FFTs, power accumulate with DC/Nyquist handled as
 * real products, scaling by 1/core_overlapped_ffts, and phase-cal folding on
 * the non-overlapped FFTs (TaskCoreIPP.cpp:633-693). */
typedef struct {
    int    fft_points;        /* N                                         */
    int    overlap;           /* fft_overlap_factor (1, 2, 4 ...)          */
    int    window;            /* 0 none, 1 cosine, 2 cosine^2              */
    int    ffts_per_spectrum; /* averaged (non-overlapped) FFTs, K         */
    int    pcal_tonebins;     /* 0 disables phase-cal                      */
    int    pcal_rotatorlen;   /* period of the pcal rotator (samples)      */
    double pcal_offset_hz;
    double sample_rate_hz;
} orc_spec_cfg;

/* core_overlapped_ffts = overlap*K - (overlap-1)   swspectrometer.cpp:231 */
int orc_spec_overlapped_ffts(const orc_spec_cfg* cfg);
/* Window w[i] computed as TaskCoreIPP::generate_windowfunction (:569-605). */
void orc_spec_window(int type, int n, float* w);
/* samples: nsamp unpacked floats.  power: nspec*(N/2+1); pcal_bins:
 * nspec*tonebins complex (may be NULL).  Returns the number of complete
 * spectra written. */
int orc_spectrometer(const float* samples, int64_t nsamp, const orc_spec_cfg* cfg,
                     float* power, orc_cf32* pcal_bins);

/* Two sources and their cross spectrum (TaskCoreIPP::doMaths with
 * num_sources = 2, num_xpols = 1, TaskCoreIPP.cpp:394-513).  power:
 * [2][nspec][N/2+1]; xpol: [nspec][N/2+1] complex (bins 1..N/2-1:
 * sum X0 conj(X1); DC and Nyquist real); pcal_bins: [2][nspec][tonebins] or
 * NULL, folded where the FFT count (advanced after every source's FFT) is a
 * multiple of the overlap.  nspec = nsamp / (N * K) spectra are written;
 * returns the number computed. */
int orc_spectrometer_xpol(const float* s0, const float* s1, int64_t nsamp, const orc_spec_cfg* cfg,
                          float* power, orc_cf32* xpol, orc_cf32* pcal_bins);

/* Phase-cal tones from folded bins: DFT of the bins scaled by 1/Nbins
 * (IPP_FFT_DIV_FWD_BY_N), first ntones outputs.  PCal.cpp:280-300. FP64. */
void orc_pcal_tones(const orc_cf32* bins, int nbins, int ntones, orc_cf32* tones);

/* FX correlator, FP32 CPU path.  Per input s and segment k: unpack N
 * samples starting at start_sample + k*N + shift[s*K + k] (2-bit, 4 per byte,
 * nchan==1), real FFT, keep channels 0..N/2-1, multiply channel c by
 * phasor[(s*K + k)*C + c] when phasor != NULL, then accumulate the lower
 * triangle V[p][c] += X_i[c]*conj(X_j[c]) with p = i*(i+1)/2 + j, j<=i,
 * through orc_addproduct_32fc_conj (architecture.h:427-433).
 * vis: P*C complex, baseline-major, accumulated (not cleared). nthreads>1
 * splits the products over pthreads. */
void orc_fx_fp32(const uint8_t* raw, int64_t bytes_per_input, int S, int N, int K,
                 int64_t start_sample, const int32_t* shift, const orc_cf32* phasor,
                 const float lut[4], int msb_first, orc_cf32* vis, int nthreads);

/* The F stage alone (used by the CPU baseline and by tests): spectra
 * out[(s*K + k)*C + c], same arithmetic as orc_fx_fp32. */
void orc_fx_fstage_fp32(const uint8_t* raw, int64_t bytes_per_input, int S, int N, int K,
                        int64_t start_sample, const int32_t* shift, const orc_cf32* phasor,
                        const float lut[4], int msb_first, orc_cf32* spectra, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
