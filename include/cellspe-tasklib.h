/*
 * cellspe-tasklib.h -- drop-in task runtime header for the GB300 engine.
 *
 * Replaces the reference's cellspe-tasklib.h (PPU section, lines 1-222).  The
 * task descriptor keeps the reference's field order, sizes and 128-byte
 * alignment (cellspe-tasklib.h:31, :36-86), so code written against the Cell
 * library compiles unchanged; the Cell SDK includes (libspe, ppu_intrinsics,
 * simdmath) are gone.  An "SPE" is now an execution slot: a host worker thread
 * with its own CUDA stream and device workspace on the GPU.  All functions
 * have C linkage (extern "C") and are exported by libcellspe_gpu.so.
 */
#ifndef CELLSPE_TASKLIB_H
#define CELLSPE_TASKLIB_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Execution slots ("SPEs").  cellspe-tasklib.h:26 */
#define CELLDSP_MAX_SPE_NR    4

#define MALLOC_QUADALIGN     7
#define ALIGNMENT_QUADALIGN  128
#define _QUAD_ALIGN  __attribute__ ((aligned(128)))

/* Task completion codes.  cellspe-tasklib.h:38-41 */
#define CELLDSP_TASK_INCOMPLETE      0xFFFF
#define CELLDSP_TASK_OK              0x0000
#define CELLDSP_TASK_GENERICERROR    0x0001
#define CELLDSP_TASK_UNKOWNCOMMAND   0x0002

/* OR-ed into CellDSPTask_t.command: the task's vectors are device pointers on
 * the engine's GPU instead of host pointers (no host<->device staging). */
#define CELLDSP_TASK_FLAG_DEVPTR     0x40000000u
#define CELLDSP_TASK_CMD_MASK        0x0000FFFFu

/* cellspe-tasklib.h:44-48 */
typedef union
{
  unsigned long long ull;
  unsigned int ui[2];
  void *p;
} Cell_addr64;

/* Sub-contexts.  cellspe-tasklib.h:50-58, plus the 2-bit unpack parameters
 * (16 bytes; the union stays within the 24 bytes the descriptor already
 * reserves before next_task, so next_task keeps its offset). */
typedef struct CellDSPParams_FFT_tt   { unsigned int nfft, log2_nfft; } CellDSPParams_FFT_t;
typedef struct CellDSPParams_Phase_tt { unsigned int argcount; float phase_start, phase_delta; } CellDSPParams_Phase_t;
typedef struct CellDSPParams_Difx_tt  { unsigned int nfft, log2_nfft, useUpperOrLower, twicenumchannels, numchannels; } CellDSPParams_Difx_t;
typedef struct CellDSPParams_Unpack_tt {
   unsigned int nsamp_lo, nsamp_hi;  /* samples per channel */
   unsigned int nchan;               /* 1, 2, 4, 8 or 16 interleaved channels */
   unsigned int format;              /* CELLSPE_LEVELS_* | CELLSPE_UNPACK_MSB_FIRST */
} CellDSPParams_Unpack_t;
typedef union CellDSKSubcontext_tt {
   CellDSPParams_FFT_t    FFT;
   CellDSPParams_Phase_t  Phase;
   CellDSPParams_Difx_t   Difx;
   CellDSPParams_Unpack_t Unpack;
} CellDSPSubcontext_t;

/* Task descriptor.  cellspe-tasklib.h:62-86 */
#define CELLDSP_MAX_NUM_IOVECTORS    8
typedef struct CellDSPTask_tt {
   unsigned int    command              _QUAD_ALIGN;
   unsigned short  completed_flag;       /* CELLDSP_TASK_* once the task ran  */
   unsigned int    tick_count;           /* device time of the task in ns,
                                            saturating at 0xFFFFFFFF          */
   unsigned int    num_input_vectors;
   Cell_addr64     inputvector_ptrs     [CELLDSP_MAX_NUM_IOVECTORS];
   unsigned int    inputvector_lengths  [CELLDSP_MAX_NUM_IOVECTORS];  /* bytes */
   unsigned int    num_output_vectors;
   Cell_addr64     outputvector_ptrs    [CELLDSP_MAX_NUM_IOVECTORS];
   unsigned int    outputvector_lengths [CELLDSP_MAX_NUM_IOVECTORS];  /* bytes */
   CellDSPSubcontext_t subcontext;
   Cell_addr64     next_task;            /* .p = NULL ends the chain */
} CellDSPTask_t _QUAD_ALIGN;

/* Behaviour flags.  cellspe-tasklib.h:164-171 */
#define CDSP_EF_RESERVED     1
#define CDSP_EF_CONTINUABLE  2
#define CDSP_EF_DEFAULT      0
#define CDSP_BEHAV_BLOCKING  1
#define CDSP_BEHAV_DEFAULT   0

/* Runtime.  cellspe-tasklib.h:122-133 (same names, arguments and return
 * conventions: 0 on success, -1 or 1 (!vecNoErr) on failure; waitTask returns
 * the task's completion code). */
int celldsp_start(void);
int celldsp_stop(void);
int celldsp_getFreeSPE(void);
int celldsp_setFreeSPE(int targetSPE);
int celldsp_startTask(int targetSPE, CellDSPTask_t * task);
int celldsp_waitTask(int targetSPE);
int celldsp_executeTask(CellDSPTask_t * task);
int celldsp_startContinuableTask(CellDSPTask_t * task, int* speID);
int celldsp_continueTask(CellDSPTask_t * task, int* speID);
int celldsp_stopContinuableTask(int* speID);
void celldsp_setBehaviour(unsigned int flags);
unsigned int celldsp_getBehaviour(void);

#ifdef __cplusplus
}  /* extern "C" */
#endif

#include "cellspe-tasklib-dsp.h"

#endif /* CELLSPE_TASKLIB_H */
