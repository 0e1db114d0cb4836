/*
 * cellspe-tasklib-dsp.h -- drop-in DSP command list and wrappers (GB300).
 *
 * Replaces the reference's cellspe-tasklib-dsp.h (lines 27-46, 79-94).  The
 * original command values 0..16 are unchanged; the GPU commands are inserted
 * before CELLDSP_TASK_SIGTERM, which stays last.
 */
#ifndef CELLSPE_TASKLIB_DSP_H
#define CELLSPE_TASKLIB_DSP_H

#include "cellspe-tasklib.h"

#ifdef __cplusplus
extern "C" {
#endif

/* types_generic.h:41-48 */
#ifndef _TYPESGENERIC_H
typedef struct { float re; float im; } fc32;
typedef fc32 cf32;
#endif

enum CellDspCommandEnum {
  CELLDSP_TASK_NOP = 0,         /* no operation                                  */
  CELLDSP_TASK_MAC,             /* out[] += in1[] * in2[]                         */
  CELLDSP_TASK_MULC,            /* out[] = in1[] * in2[]                          */
  CELLDSP_TASK_ADDC,            /* out[] = in1[] + in2[]                          */
  CELLDSP_TASK_IOTEST,          /* writes {0.1, 2.3, 4.5, 6.7} to out0            */
  CELLDSP_TASK_IOBENCH,         /* Cell DMA benchmark: accepted, no work          */
  CELLDSP_TASK_FFT_INIT,        /* prepare continuable FFT (keeps the slot)       */
  CELLDSP_TASK_FFT_FREE,        /* release continuable FFT                        */
  CELLDSP_TASK_FFT_EXEC,        /* forward C2C FFT of nfft points                 */
  CELLDSP_TASK_FFT_EXEC_DYN,    /* same, any nfft without init                    */
  CELLDSP_TASK_SINCOS,          /* interleaved {cos, sin} of in0                  */
  CELLDSP_TASK_SINCOS_NORM,     /* same with phases in turns (1.0 = 2 pi)         */
  CELLDSP_TASK_SINCOS_GENERTR,  /* {cos, sin}(phase_start + n * phase_delta)      */
  CELLDSP_TASK_UNPACK,          /* 2-bit raw -> float planes (subcontext.Unpack)  */
  CELLDSP_TASK_RUNALL,          /* Cell timing skeleton: accepted, no work        */
  CELLDSP_TASK_DMASIMULATION,   /* Cell DMA-list test: accepted, no work          */
  CELLDSP_TASK_DIFXPROCESS,     /* FFT + fractional-sample multiply + autocorr    */
  /* ---- GB300 engine commands ---- */
  CELLDSP_TASK_MAC_CONJ,        /* out[] += in1[] * conj(in2[])                   */
  CELLDSP_TASK_RFFT,            /* batched R2C: in0 N reals per row -> N/2+1 bins */
  CELLDSP_TASK_FX_CORRELATE,    /* in0 cellspe_fx_params, in1 raw, in2 delay poly
                                   (optional); out0 visibilities                  */
  CELLDSP_TASK_SPECTROMETER,    /* in0 cellspe_spec_params, in1 raw; out0 power,
                                   out1 pcal bins, out2 pcal tones (optional)     */
  CELLDSP_TASK_XMAC,            /* in0 cellspe_xmac_params, in1 spectra; out0 vis */
  CELLDSP_TASK_SIGTERM          /* terminate (always keep as last entry)          */
};

/* PPU-side wrappers.  cellspe-tasklib-dsp.h:79-94 (header signatures). */
int speNOP(void);
int speRunAllCheck(void);
int speIOCheck(void);
int speIOSimulation(void);
int speIOBench(void* buffer, unsigned int bufbytes, int spes);
int speIOBenchStreamed(void* buffer, unsigned int bufbytes, int spes, int stream_length);
int speAddProduct_32fc(fc32 * src, fc32 * src2, fc32 * accumulator, int length);
int speFFT_init(int fft_len, int* speID);
int speFFT_exec(void* in, void* out, int fft_len, int* speID);
int speFFT_destroy(int* speID);
int speFFT_singleexec(void* in, void* out, int fft_len);
int speDIFX_process(void* sincosrotdone, void* complexfracmult, void* fftoutJ, void* conjfftoutJ, void* autocorr,
                    int nfft, int twicenumchannels, int useUpperOrLower);
int speSinCosGenerator(float startphase, float increment, fc32* cos_sin_out, int numiter);
int speSinCosAccurate(float * argument, cf32 * cos_sin_out, int argumentcount);
int speSinCosAccurateNorm(float * normalizedargument, cf32 * cos_sin_out, int argumentcount);

#ifdef __cplusplus
}  /* extern "C" */
#endif

#endif /* CELLSPE_TASKLIB_DSP_H */
