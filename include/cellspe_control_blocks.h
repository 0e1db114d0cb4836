/* The reference's Cell control blocks, accepted by the GB300 engine.
 *
 * The reference hands its SPE programs a control block in main memory: the
 * minicorrelator one `control_block` per SPE (minicorrelator/minicorrelator.h:
 * 107-119, filled by minicorrelator_ppu.c:131-148), the Cell spectrometer
 * one `control_block_t` per task (spectrometer/src/Cell/cell_spectrometer.h:
 * 104-115, filled by TaskCoreCell.cpp:43-48, 76-79).  The types below keep
 * the reference's member order, sizes and 128-byte alignment, so a PPU-side
 * caller fills them exactly as before; the entry points run what the SPE
 * programs ran, on the GPU.
 *
 * Return value: 0 on success or a CELLSPE_ERR_* code (cellspe_gpu.h), with
 * cellspe_last_error() describing the failure.
 */
#ifndef CELLSPE_CONTROL_BLOCKS_H
#define CELLSPE_CONTROL_BLOCKS_H

#ifdef __cplusplus
extern "C" {
#endif

#define CELLSPE_CB_ALIGN __attribute__((aligned(128)))

/* 64-bit effective address (minicorrelator.h:68-72, cell_spectrometer.h:97-101) */
typedef union {
    unsigned long long ull;
    unsigned int ui[2];
    void* p;
} addr64;

/* minicorrelator.h:107-119, "HARD-CODED 6 STATION EXPERIMENT" */
typedef struct _control_block {
    addr64 rawdata_src CELLSPE_CB_ALIGN;   /* this SPE's station: ffts_total x 256 bytes of 2-bit samples */
    addr64 autocorrelation_out;            /* [blocks][Re x 1024 | Im x 1024] float                       */
    addr64 baselines_out[15];              /* same layout per baseline slot                               */
    addr64 fmultipliers_src;               /* placeholder oscillator multipliers (not used, see below)    */
    addr64 syncline;                       /* Cell SPE synchronisation line (not used)                    */
    int spe_num;                           /* rank of this SPE = its station                              */
    int num_spes;                          /* 6                                                           */
    unsigned int ffts_total;               /* 1024-sample FFT buffers per station                         */
    unsigned int ffts_to_integrate;        /* FFT buffers per output block (even)                         */
    addr64 spe_ls_listOnPPU;               /* Cell local-store map (not used)                             */
    addr64 spe_sig_listOnPPU;              /* Cell signal map (not used)                                  */
} control_block CELLSPE_CB_ALIGN;

/* cell_spectrometer.h:104-115 */
typedef struct control_block_tt {
    unsigned int rank CELLSPE_CB_ALIGN;
    unsigned int terminate_flag;           /* 1: release the task's state and return                       */
    unsigned int fft_points;               /* N, a power of two, 32 .. 32768                               */
    unsigned int fft_points_log2;
    unsigned int overlap_factor;           /* FFTs advance by raw bytes of one FFT / overlap_factor        */
    unsigned int integrate_ffts;           /* K: FFTs per spectrum                                         */
    unsigned int samples_per_rawbyte;      /* 1: 8-bit offset binary (byte - 127.5), 4: 2-bit             */
    addr64 rawif_src;                      /* raw IF bytes (host memory)                                   */
    unsigned int rawif_bytecount;
    addr64 spectrum_dst;                   /* spectra: [spectra][N] x {power, 0} floats (host memory)      */
} control_block_t CELLSPE_CB_ALIGN;

/* The minicorrelator's SPE job for all num_spes control blocks at once
 * (minicorrelator_spu.c:255-481): station s = cbs[s].spe_num reads
 * ffts_total x 256 bytes from its rawdata_src.  Each time period of the
 * reference (two 1024-sample FFT buffers, 512 bytes) is one 2048-sample real
 * segment here; its 1024 channels fill the reference's N_FFT-bin result
 * buffers.  Every ffts_to_integrate buffers (ffts_to_integrate / 2 segments)
 * block b is written (minicorrelator_spu.c:835-866): the autocorrelation of
 * station s to cbs[s].autocorrelation_out and, for m = 0, 1, 2, the cross
 * product X_s conj(X_o), o = (s + {1, 3, 4}[m]) mod 6, to
 * cbs[s].baselines_out[s + 6 m] when that slot is below 15 -- the reference's
 * slot assignment (minicorrelator_spu.c:302-304, 841-858), whose three
 * duplicated pairs are kept.  Each block is Re x 1024 then Im x 1024 floats
 * at byte offset b x 8192, the FP32 sums over its segments.  Samples are
 * 2-bit offset binary, LSB first (CELLSPE_LEVELS_OFFSET_BINARY: the
 * reference's lookup table is a placeholder, minicorrelator_spu.c:314-317);
 * the placeholder fringe multipliers (fmultipliers_src, sincos_fast) and
 * the Cell-only members are not used.  Needs num_spes == 6 (the struct holds
 * 15 baseline slots), the same ffts_total and ffts_to_integrate in every
 * block, spe_num a permutation of 0..5, host pointers. */
int cellspe_minicorrelator_run(const control_block* cbs, int num_spes);

/* The Cell spectrometer's SPE task (spectrometer_spu.c:96-205), one call per
 * mailbox start.  *state holds what the SPE keeps between tasks (its FFT
 * size, window, the partly integrated spectrum and its FFT count): NULL on
 * the first call, set by it; a call with terminate_flag != 0 releases it
 * (sets *state to NULL) and returns 0.
 *
 * A task reads FFT f from byte f x d of rawif_src, d = (N / spr) /
 * overlap_factor, for f < floor(rawif_bytecount / d) - 1 (the reference's
 * loop bound; FFTs that would read past the buffer, which the SPE's DMA
 * does for overlap_factor > 2, are not done), decodes N samples (spr = samples_per_rawbyte = 1: byte -
 * 127.5 as unpack_windowed_to_fft; 4: 2-bit LSB-first codes through
 * `levels4`, NULL for CELLSPE_LEVELS_TWOBIT), weights them by sin^2(pi i /
 * (N - 1)) (calc_cos_window_function), adds |X[k]|^2 / K of the N-point
 * real FFT into the running spectrum and, each time K FFTs are in, writes
 * the spectrum to the next N x {power, 0} slot of spectrum_dst (bins k and
 * N - k carry the same power) and starts a new one.  A partial spectrum
 * carries over to the next call, as on the SPE.  Scaling is 1 / K (the SPE
 * scales each FFT by 1 / K before squaring, i.e. 1 / K^2; the engine's
 * spectrometers average).  stats (optional): [0] device time in ns of the
 * task, [1] spectra written, [2] FFTs done -- what the SPE reports through
 * its mailbox (TaskCoreCell.cpp:94-116). */
int cellspe_cell_spectrometer_task(void** state, const control_block_t* cb, const float* levels4,
                                   unsigned int stats[3]);

#ifdef __cplusplus
}
#endif

#endif /* CELLSPE_CONTROL_BLOCKS_H */
