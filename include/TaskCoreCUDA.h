/* TaskCoreCUDA -- the swspectrometer's computing core on the GPU.
 *
 * Drop-in for the spectrometer's platform core (TaskCoreIPP,
 * spectrometer/src/IA-32/TaskCoreIPP.h) behind the TaskCore interface
 * (spectrometer/src/TaskCore.h:36-89).  Select it in TaskDispatcher.h
 * (spectrometer/src/TaskDispatcher.h:26-39) with
 *
 *     #include "TaskCoreCUDA.h"
 *     #define Platform_TaskCore TaskCoreCUDA
 *
 * add TaskCoreCUDA.cpp to the spectrometer's sources and link
 * libcellspe_gpu.so.  TaskDispatcher then drives it unchanged:
 * prepare(settings) once per core, and per raw buffer run() (returns at once),
 * join() (complete spectra in the core's output buffers, or -1),
 * combineResults() when one spectrum spans several raw buffers, finalize().
 *
 * The maths is TaskCoreIPP::doMaths (TaskCoreIPP.cpp:394-513) on the GPU:
 * 2-bit unpack of the chosen channel of each source, window, overlapped real
 * FFTs, |X|^2 accumulation with DC and Nyquist from the real parts, the
 * cross-polarisation product of two sources, the phase-cal fold, scaling by
 * 1/core_overlapped_ffts.  Sub-spectra are added on the GPU in
 * combineResults.  Supported inputs: 2 bits per sample, 4, 8 or 16 channels,
 * sourceformat RawSigned / RawUnsigned (TwoBitUnpacker, either channel
 * order), Mark5B (payloads with headers removed, Mark5BUnpacker's levels)
 * and Mk5B (mark5access levels); windows None, Cosine, Cosine2, Hamming,
 * Hann, Blackman; one or two sources with at most one cross product.
 * prepare() reports anything else on stderr and join() then returns -1.
 *
 * The core compiles against the spectrometer's own TaskCore.h / Settings.h /
 * Buffer.h, or against the stand-ins in cellspe-tasklib_gb300/taskcore/compat
 * where that tree is absent (same layouts). */
#ifndef TASKCORE_CUDA_H
#define TASKCORE_CUDA_H

#include <condition_variable>
#include <mutex>
#include <thread>

#include "TaskCore.h"

class TaskCoreCUDA : public TaskCore
{
public:
   explicit TaskCoreCUDA(int rank);
   TaskCoreCUDA();
   ~TaskCoreCUDA() override;

   void prepare(swspect_settings_t* settings) override;
   int run(Buffer** inbuf, Buffer** outbuf, Buffer** xpolbuf, Buffer** pcalbuf) override;
   int join() override;
   int finalize() override;
   int combineResults(Buffer** outbuf, Buffer** pcalbuf) override;
   void resetBuffer(Buffer* buf) override;

   /* The text of the last failure of this core ("" when none). */
   const char* lastError() const { return error_; }

private:
   void worker();
   int compute();
   int fail(const char* msg);
   bool grow(void** p, size_t* cap, size_t bytes);
   void releaseDevice();

   int rank_ = 0;
   swspect_settings_t* cfg_ = nullptr;
   bool ok_ = false;                 /* prepare() accepted the settings */
   int levels_ = 0;                  /* CELLSPE_LEVELS_* */
   int nsub_ = 0;                    /* channels interleaved per source */
   int chan_[2] = {0, 0};            /* subband index each source uses */
   int nsrc_ = 0, nxpol_ = 0;
   int K_ = 0;                       /* non-overlapped FFTs per (sub-)spectrum */

   /* device memory (grown on demand, kept between runs) */
   void* d_raw_[2] = {nullptr, nullptr};
   size_t raw_cap_[2] = {0, 0};
   void* d_power_ = nullptr;
   size_t power_cap_ = 0;
   void* d_xpol_ = nullptr;
   size_t xpol_cap_ = 0;
   void* d_pcal_ = nullptr;
   size_t pcal_cap_ = 0;
   void* d_acc_ = nullptr;
   size_t acc_cap_ = 0;

   /* results of the last run, on the device: per source the first spectrum */
   int nspec_ = 0;
   float* own_power_[2] = {nullptr, nullptr};
   float* own_xpol_ = nullptr;
   float* own_pcal_[2] = {nullptr, nullptr};
   bool have_results_ = false;

   /* the run handed to the worker thread */
   Buffer** in_ = nullptr;
   Buffer** out_ = nullptr;
   Buffer** xpol_ = nullptr;
   Buffer** pcal_ = nullptr;
   std::thread thread_;
   std::mutex mu_;
   std::condition_variable cv_;
   enum Stage { IDLE, QUEUED, DONE, QUIT } stage_ = IDLE;
   int result_ = 0;
   char error_[256] = {0};
};

#endif /* TASKCORE_CUDA_H */
