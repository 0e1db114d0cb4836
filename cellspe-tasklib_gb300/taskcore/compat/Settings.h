// Stand-in for the swspectrometer's settings block (spectrometer/src/
// Settings.h:37-159), used where that source tree is not on the include path.
// The enums and swspect_settings_t keep the original's members, types and
// order, so a settings block filled in by a swspectrometer build has the same
// layout; the sources, sinks and log objects it points to are only declared.
#ifndef SETTINGS_H
#define SETTINGS_H

#include <cstddef>
#include <string>
#include <vector>

#include "Buffer.h"

typedef float               swsfloat_t;
typedef unsigned long long  swsint64_t;

typedef struct _swscomplex_t {
   swsfloat_t re, im;
} swscomplex_t;

enum WindowFunctionType { None, Cosine, Cosine2, Hamming, Hann, Blackman };
enum OutputFormat { Ascii, Binary };
enum InputFormat  { Unknown=-1, RawSigned, RawUnsigned, Mark5B, iBOB, VDIF, VLBA, MKIV, Mk5B, Maxim };

class DataSink;
class DataSource;
class LogFile;
class TeeStream;

typedef struct swspect_settings_tt {
   // calculation parameters (command line / INI)
   int num_cores;                      // worker cores
   size_t fft_points;                  // FFT length N
   swsfloat_t fft_integ_seconds;       // integration time of one spectrum
   int fft_overlap_factor;             // hop = N / overlap
   WindowFunctionType wf_type;         // window
   int bits_per_sample;                // raw bits per sample
   bool channelorder_increasing;       // channel 0 in the low bits of the first byte
   int seconds_to_skip;
   int source_channels;                // channels interleaved in a source
   int use_channel_file1;              // channel used from source 1 (0-based once parsed)
   int use_channel_file2;              // channel used from source 2
   swsfloat_t samplingfreq;            // Hz
   swsfloat_t pcaloffsethz;            // phase-cal comb offset
   swsfloat_t pcalharmonicshz;         // phase-cal comb spacing
   size_t max_rawbuf_size;
   bool extract_PCal;
   bool calc_Xpol;
   bool costas_loop;
   bool use_live_plot;
   std::string basefilename1_pattern;
   std::string basefilename2_pattern;

   // sources and sinks
   std::vector<DataSource*> sources;
   std::vector<DataSink*>   sinks;
   std::vector<DataSink*>   pcalsinks;
   int num_sources;
   int num_sinks;
   int num_xpols;
   InputFormat  sourceformat;
   std::string  sourceformat_str;
   OutputFormat sinkformat;

   // buffers: [core][double buffer][source], [core][source], [core][xpol], [core][source]
   Buffer**** rawbuffers;
   Buffer***  outbuffers;
   Buffer***  outbuffersXpol;
   Buffer***  outbuffersPCal;

   // derived parameters
   std::string basefilename1;
   std::string basefilename2;
   swsfloat_t dt;
   swsfloat_t df;
   int averaged_ffts;                  // non-overlapped FFTs per spectrum
   int averaged_overlapped_ffts;
   int fft_overlap_points;             // N / overlap
   int fft_ssb_points;                 // N/2 + 1
   double rawbytes_per_channelsample;  // bits * source_channels / 8
   size_t raw_fullfft_bytes;
   size_t raw_overlap_bytes;
   size_t fft_bytes;
   size_t fft_bytes_ssb;               // (N/2 + 1) floats
   size_t fft_bytes_xpol;              // 2 * fft_bytes_ssb
   size_t rawbuf_size;
   int max_spectra_per_buffer;
   int max_specffts_per_buffer;
   int max_buffers_per_spectrum;
   int core_overlapped_ffts;           // overlapped FFTs a core adds into one spectrum
   int core_averaged_ffts;             // non-overlapped FFTs a core covers per spectrum
   int pcal_tonebins;
   int pcal_rotatorlen;
   int pcal_pulses;
   int pcal_pulses_per_fft;
   size_t pcal_result_bytes;           // tonebins complex floats

   // logs
   LogFile* logIO;
   LogFile* log;
   TeeStream* tlog;
} swspect_settings_t;

#endif // SETTINGS_H
