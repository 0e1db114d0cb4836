/* In-memory spectrometer run through TaskCoreCUDA cores, driven the way the
 * swspectrometer's TaskDispatcher drives its platform cores.
 *
 * cellspe_taskcore_spectrometer derives the run's settings from `c` as
 * swspectrometer does from its INI file (spectrometer/src/swspectrometer.cpp:
 * 164-230: averaged FFTs, raw buffer size split over the cores and halved for
 * double buffering, spectra per buffer or buffers per spectrum,
 * core_overlapped_ffts, phase-cal bins and rotator length), creates
 * num_cores TaskCoreCUDA cores with double-buffered raw buffers, and runs
 * TaskDispatcher::run's cycle (spectrometer/src/TaskDispatcher.cpp:92-243):
 * start every core on its buffers, read the next buffers, join each core in
 * order and either write its spectra or add them into the common spectra with
 * combineResults, writing a common spectrum once max_buffers_per_spectrum
 * sub-spectra are in.  The sources are the recordings src0 (and src1 with
 * two sources), `bytes` bytes each; every buffer that receives data is
 * processed (the run ends when core 0's next buffers come back empty).  The
 * sinks are byte streams: auto spectra of source 0 and 1, the cross spectrum,
 * phase-cal bins of source 0 and 1, written as the dispatcher writes them
 * (each write appends the buffer's current length).
 *
 * Returns 0, or -1 with the text in cellspe_taskcore_last_error(). */
#ifndef CELLSPE_TASKCORE_H
#define CELLSPE_TASKCORE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int    num_cores;               /* NumCPUCores: TaskCoreCUDA instances          */
    int    fft_points;              /* DFTLength                                    */
    double integ_seconds;           /* FFTIntegrationTimeSec                        */
    int    overlap;                 /* FFToverlapFactor                             */
    int    window;                  /* WindowFunction: 0 None .. 5 Blackman         */
    int    source_channels;         /* SourceChannels                               */
    int    channel1, channel2;      /* UseFile1Channel / UseFile2Channel (1-based)  */
    int    channelorder_increasing; /* ChannelOrderIncreasing                       */
    int    sourceformat;            /* InputFormat: 0 RawSigned, 1 RawUnsigned,
                                     * 2 Mark5B, 7 Mk5B                             */
    double samplingfreq;            /* 2 x BandwidthHz                              */
    int    extract_pcal;            /* ExtractPCal                                  */
    double pcal_offset_hz;          /* PCalOffsetHz                                 */
    double pcal_harmonics_hz;       /* PCalHarmonicsHz (comb spacing)               */
    int    num_sources;             /* 1 or 2 recordings                            */
    int    calc_xpol;               /* cross product of two sources                 */
    long long max_rawbuf_bytes;     /* MaxSourceBufferMB x 2^20 / 2                 */
} cellspe_taskcore_config;

/* sinks: [0] auto source 0, [1] auto source 1, [2] cross, [3] pcal source 0,
 * [4] pcal source 1; sink_cap[i] bytes available at sink[i] (NULL = unused),
 * sink_bytes[i] receives the bytes written.  spectra_written receives the
 * dispatcher's spectrum count. */
int cellspe_taskcore_spectrometer(const cellspe_taskcore_config* c, const void* src0, const void* src1,
                                  long long bytes, void* const sink[5], const long long sink_cap[5],
                                  long long sink_bytes[5], long long* spectra_written);
const char* cellspe_taskcore_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* CELLSPE_TASKCORE_H */
