/* Multi-tone phase-cal extraction on the GPU: the reference's PCal library
 * (spectrometer/src/IA-32/PhaseCal/PCal.h:46-190, PCal.cpp:92-690).
 *
 * An extractor folds a continuous real sample stream, handed over in pieces
 * of any length, onto N_bins bins (sample n of the stream, counted from the
 * sample offset, lands in bin n mod N_bins), optionally mixed down by the
 * phase-cal offset first, and at the end takes a DFT of the bins (divided by
 * N_bins, IPP_FFT_DIV_FWD_BY_N) and picks the tone bins.  PCal::getNew's
 * choice of method is kept (cellspe_pcal_new):
 *   offset 0                              -> Trivial      (PCal.cpp:203-316)
 *   No % Np == 0, No = fs / gcd(offset, fs), Np = fs / gcd(spacing, fs)
 *                                         -> ImplicitShift (PCal.cpp:521-690)
 *   otherwise                             -> Shifting     (PCal.cpp:321-510)
 * with fs = 2 x bandwidth.  Trivial:  N_bins = Np, N_tones = floor(bw /
 * spacing), tones = DFT bins 0 .. N_tones-1.  Shifting: N_bins = Np, samples
 * times exp(-2 pi i offset n / fs) (period No), tones = bins n x step, step =
 * floor(N_bins spacing / fs).  ImplicitShift: N_bins = No, no mixing, tones =
 * bins floor(N_bins offset / fs) + n x step.  Shifting and ImplicitShift have
 * N_tones = floor((bw - offset) / spacing) + 1; tones whose bin would be
 * >= N_bins are left unwritten, as in the reference.
 *
 * Deviations (each a reference defect, not reproduced): the extractors start
 * at the getNew sample offset (the reference leaves its bin index
 * uninitialised until adjustSampleOffset); Shifting counts every sample (the
 * reference's per-period loop adds rotator-period / N_bins whole pulses and
 * drops the rest of each period, which happens exactly when getNew picks
 * Shifting, PCal.cpp:437-447).
 *
 * Accumulation is FP32 on the device (the reference's ippsAdd_32f/32fc);
 * the final DFT of the picked bins is evaluated per tone on the device.
 * Return values: 0 or CELLSPE_ERR_* (cellspe_gpu.h), cellspe_last_error().
 */
#ifndef CELLSPE_PCAL_H
#define CELLSPE_PCAL_H

#ifdef __cplusplus
extern "C" {
#endif

#define CELLSPE_PCAL_TRIVIAL        0
#define CELLSPE_PCAL_SHIFTING       1
#define CELLSPE_PCAL_IMPLICIT_SHIFT 2

typedef struct cellspe_pcal cellspe_pcal;

/* PCal::getNew(bandwidth_hz, pcal_spacing_hz, pcal_offset_hz, sampleoffset);
 * NULL on failure (bandwidth and spacing must be positive whole numbers of
 * Hz, offset >= 0, N_bins <= 2^28). */
cellspe_pcal* cellspe_pcal_new(double bandwidth_hz, double pcal_spacing_hz, int pcal_offset_hz,
                               unsigned long long sampleoffset);
void cellspe_pcal_free(cellspe_pcal* pc);
/* CELLSPE_PCAL_* of the method getNew picked */
int cellspe_pcal_kind(const cellspe_pcal* pc);
/* getLength(): tones in the result; getNBins(): folding bins */
int cellspe_pcal_length(const cellspe_pcal* pc);
long long cellspe_pcal_nbins(const cellspe_pcal* pc);
/* getSeconds(): samples integrated / fs */
double cellspe_pcal_seconds(const cellspe_pcal* pc);
/* clear(): bins and sample count to zero, not finalised (PCal.cpp:264-270) */
int cellspe_pcal_clear(cellspe_pcal* pc);
/* adjustSampleOffset(sampleoffset): the next sample is sample `sampleoffset`
 * of the subintegration (PCal.cpp:278-282, 397-401, 588-591) */
int cellspe_pcal_adjust_sample_offset(cellspe_pcal* pc, unsigned long long sampleoffset);
/* extractAndIntegrate(samples, len): any len >= 0; CELLSPE_ERR_ARG after
 * cellspe_pcal_final until cellspe_pcal_clear (the reference returns false) */
int cellspe_pcal_extract(cellspe_pcal* pc, const float* samples, long long len, int memory);
/* getFinalPCal(out): writes the tones (complex64, cellspe_pcal_length of
 * them, host memory) and returns the samples integrated, or -CELLSPE_ERR_* */
long long cellspe_pcal_final(cellspe_pcal* pc, void* out);

#ifdef __cplusplus
}
#endif

#endif /* CELLSPE_PCAL_H */
