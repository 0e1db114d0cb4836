// In-memory spectrometer run through TaskCoreCUDA cores (cellspe_taskcore.h).
//
// The settings are derived the way swspectrometer.cpp:164-230 derives them
// from its INI file, the buffers are laid out as swspectrometer.cpp:363-413
// lays them out ([core][double buffer][source] raw buffers, [core][source]
// output buffers), and the cycle is TaskDispatcher::run's
// (TaskDispatcher.cpp:92-243).  The code is this library's own; the order of
// the calls into the cores is the reference dispatcher's, because that order
// is the plug-in contract TaskCoreCUDA has to meet.
#include "cellspe_taskcore.h"

#include <algorithm>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "Buffer.h"
#include "TaskCoreCUDA.h"

namespace {

thread_local std::string t_err;

int set_err(const std::string& m)
{
    t_err = m;
    return -1;
}

long long gcd_ll(long long a, long long b)
{
    while (b) {
        long long t = a % b;
        a = b;
        b = t;
    }
    return a;
}

// A recording read in raw-buffer sized pieces (FileSource::read for
// headerless data: as many bytes as the buffer holds, fewer at the end).
struct MemSource {
    const unsigned char* p;
    long long left;
    void read(Buffer* b)
    {
        const long long n = std::min<long long>((long long)b->getAllocated(), left);
        if (n > 0) std::memcpy(b->getData(), p, (size_t)n);
        b->setLength((size_t)std::max<long long>(n, 0));
        p += std::max<long long>(n, 0);
        left -= std::max<long long>(n, 0);
    }
};

// A sink that appends each written buffer's current length.
struct MemSink {
    unsigned char* p;
    long long cap, used;
    bool write(Buffer* b)
    {
        const long long n = (long long)b->getLength();
        if (!p || used + n > cap) return false;
        std::memcpy(p + used, b->getData(), (size_t)n);
        used += n;
        return true;
    }
};

}  // namespace

extern "C" const char* cellspe_taskcore_last_error(void) { return t_err.c_str(); }

extern "C" int cellspe_taskcore_spectrometer(const cellspe_taskcore_config* c, const void* src0, const void* src1,
                                             long long bytes, void* const sink[5], const long long sink_cap[5],
                                             long long sink_bytes[5], long long* spectra_written)
{
    if (!c || !src0 || bytes <= 0 || !sink || !sink_cap || !sink_bytes) return set_err("taskcore: bad arguments");
    if (c->num_cores < 1 || c->num_sources < 1 || c->num_sources > 2 || (c->num_sources == 2 && !src1))
        return set_err("taskcore: num_cores >= 1 and one or two sources");
    if (c->fft_points < 16 || c->overlap < 1 || c->samplingfreq <= 0 || c->max_rawbuf_bytes <= 0)
        return set_err("taskcore: bad FFT, overlap, sampling or buffer settings");

    // ---- settings (swspectrometer.cpp:164-230) -----------------------------
    swspect_settings_t set;
    set.num_cores = c->num_cores;
    set.fft_points = (size_t)c->fft_points;
    set.fft_integ_seconds = (swsfloat_t)c->integ_seconds;
    set.fft_overlap_factor = c->overlap;
    set.wf_type = (WindowFunctionType)c->window;
    set.bits_per_sample = 2;
    set.channelorder_increasing = c->channelorder_increasing != 0;
    set.seconds_to_skip = 0;
    set.source_channels = c->source_channels;
    set.use_channel_file1 = c->channel1 - 1;                 // 1..CH in the INI
    set.use_channel_file2 = c->channel2 - 1;
    set.samplingfreq = (swsfloat_t)c->samplingfreq;
    set.pcaloffsethz = (swsfloat_t)c->pcal_offset_hz;
    set.pcalharmonicshz = (swsfloat_t)c->pcal_harmonics_hz;
    set.max_rawbuf_size = (size_t)c->max_rawbuf_bytes;
    set.extract_PCal = c->extract_pcal != 0;
    set.calc_Xpol = c->calc_xpol != 0;
    set.costas_loop = false;
    set.use_live_plot = false;
    set.num_sources = c->num_sources;
    set.num_xpols = (c->num_sources == 2 && c->calc_xpol) ? 1 : 0;
    set.num_sinks = set.num_sources + set.num_xpols;
    set.sourceformat = (InputFormat)c->sourceformat;
    set.sinkformat = Binary;
    set.rawbuffers = nullptr;
    set.outbuffers = set.outbuffersXpol = set.outbuffersPCal = nullptr;
    set.logIO = set.log = nullptr;
    set.tlog = nullptr;

    set.dt = 1.0f / set.samplingfreq;
    set.df = set.samplingfreq / (swsfloat_t)set.fft_points;
    set.averaged_ffts = (int)((set.samplingfreq * set.fft_integ_seconds) / (swsfloat_t)set.fft_points);
    set.averaged_overlapped_ffts = 0;
    set.fft_overlap_points = (int)set.fft_points / set.fft_overlap_factor;
    set.fft_ssb_points = (int)set.fft_points / 2 + 1;
    set.rawbytes_per_channelsample = (set.bits_per_sample * set.source_channels) / 8.0;
    set.raw_fullfft_bytes = (size_t)(set.fft_points * set.rawbytes_per_channelsample);
    set.raw_overlap_bytes = (size_t)(set.fft_overlap_points * set.rawbytes_per_channelsample);
    set.fft_bytes = set.fft_points * sizeof(swsfloat_t);
    set.fft_bytes_ssb = (size_t)set.fft_ssb_points * sizeof(swsfloat_t);
    set.fft_bytes_xpol = 2 * set.fft_bytes_ssb;
    if (set.averaged_ffts < 1) return set_err("taskcore: integration shorter than one FFT");

    if (set.extract_PCal) {
        if (c->pcal_harmonics_hz <= 0) return set_err("taskcore: phase-cal needs a comb spacing");
        const long long fs = (long long)set.samplingfreq, off = (long long)set.pcaloffsethz;
        set.pcal_tonebins = (int)(set.samplingfreq / set.pcalharmonicshz);
        // fs / gcd(fs, offset); the reference divides by zero for a zero offset,
        // whose rotator is one comb period
        set.pcal_rotatorlen = off == 0 ? set.pcal_tonebins : (int)(fs / gcd_ll(fs, off));
        set.pcal_pulses = set.pcal_rotatorlen / std::max(set.pcal_tonebins, 1);
        set.pcal_result_bytes = (size_t)set.pcal_tonebins * 2 * sizeof(float);
        set.pcal_pulses_per_fft = (int)set.fft_points / set.pcal_rotatorlen;
        if (set.fft_points % (size_t)set.pcal_rotatorlen) set.extract_PCal = false;   // as the reference warns
    }
    if (!set.extract_PCal) {
        set.pcal_tonebins = set.pcal_rotatorlen = set.pcal_pulses = set.pcal_pulses_per_fft = 0;
        set.pcal_result_bytes = 0;
    }

    set.max_rawbuf_size = set.max_rawbuf_size / set.num_cores;
    size_t tent = set.raw_fullfft_bytes * set.averaged_ffts;
    if (tent > set.max_rawbuf_size) {
        set.max_spectra_per_buffer = 0;
        set.max_specffts_per_buffer = 1;
        set.max_buffers_per_spectrum = set.averaged_ffts;
        tent = set.raw_fullfft_bytes;
        while (tent <= set.max_rawbuf_size && (set.max_buffers_per_spectrum % 2) == 0) {
            tent *= 2;
            set.max_buffers_per_spectrum /= 2;
            set.max_specffts_per_buffer *= 2;
        }
    } else {
        set.max_spectra_per_buffer = 1;
        set.max_specffts_per_buffer = set.averaged_ffts;
        set.max_buffers_per_spectrum = 0;
        while (2 * tent <= set.max_rawbuf_size) {
            tent *= 2;
            set.max_spectra_per_buffer *= 2;
        }
    }
    set.rawbuf_size = tent;
    set.core_averaged_ffts = set.max_specffts_per_buffer;
    set.core_overlapped_ffts = set.fft_overlap_factor * set.max_specffts_per_buffer - (set.fft_overlap_factor - 1);

    // ---- buffers (swspectrometer.cpp:363-413) ------------------------------
    const int ncores = set.num_cores, nsrc = set.num_sources;
    std::vector<std::unique_ptr<Buffer>> keep;
    auto make = [&](size_t n) {
        keep.emplace_back(new Buffer(n));
        return keep.back().get();
    };
    std::vector<std::vector<std::vector<Buffer*>>> raw(ncores, std::vector<std::vector<Buffer*>>(2));
    std::vector<std::vector<Buffer*>> out(ncores), xpol(ncores), pcal(ncores);
    const size_t nmax = (size_t)std::max(set.max_spectra_per_buffer, 1);
    for (int k = 0; k < ncores; k++) {
        for (int b = 0; b < 2; b++)
            for (int s = 0; s < nsrc; s++) raw[k][b].push_back(make(set.rawbuf_size));
        for (int s = 0; s < nsrc; s++) out[k].push_back(make(nmax * set.fft_bytes_ssb));
        for (int x = 0; x < set.num_xpols; x++) xpol[k].push_back(make(nmax * set.fft_bytes_xpol));
        for (int s = 0; s < nsrc; s++) pcal[k].push_back(make(std::max<size_t>(nmax * set.pcal_result_bytes, 8)));
    }

    MemSource src[2] = {{(const unsigned char*)src0, bytes}, {(const unsigned char*)src1, nsrc == 2 ? bytes : 0}};
    MemSink snk[5];
    for (int i = 0; i < 5; i++) snk[i] = {(unsigned char*)sink[i], sink[i] ? sink_cap[i] : 0, 0};
    auto auto_sink = [&](int s) -> MemSink& { return snk[s]; };
    auto pcal_sink = [&](int s) -> MemSink& { return snk[3 + s]; };
    bool sink_ok = true;

    // ---- TaskDispatcher: prefill, cores, common buffers ---------------------
    for (int k = 0; k < ncores; k++)
        for (int s = 0; s < nsrc; s++) src[s].read(raw[k][0][s]);
    std::vector<std::unique_ptr<TaskCoreCUDA>> cores;
    for (int k = 0; k < ncores; k++) {
        cores.emplace_back(new TaskCoreCUDA(k));
        cores.back()->prepare(&set);
    }
    std::vector<Buffer*> common_spec, common_pcal;
    const size_t peak = std::max(set.fft_bytes_xpol, set.fft_bytes_ssb);
    for (int i = 0; i < set.num_sinks; i++) {
        common_spec.push_back(make(peak));
        common_spec.back()->setLength(peak);
        cores[0]->resetBuffer(common_spec.back());
    }
    for (int s = 0; s < nsrc; s++) {
        common_pcal.push_back(make(std::max<size_t>(set.pcal_result_bytes, 8)));
        common_pcal.back()->setLength(set.pcal_result_bytes);
        cores[0]->resetBuffer(common_pcal.back());
    }

    long long total = 0;
    int db = 0, combined = 0;
    int rc = 0;
    for (;;) {
        for (int k = 0; k < ncores; k++)
            cores[k]->run(raw[k][db].data(), out[k].data(), xpol[k].data(), pcal[k].data());
        for (int k = 0; k < ncores; k++)
            for (int s = 0; s < nsrc; s++) src[s].read(raw[k][(db + 1) % 2][s]);
        for (int k = 0; k < ncores; k++) {
            const int n = cores[k]->join();
            if (n < 0) {
                rc = set_err(std::string("taskcore: ") + cores[k]->lastError());
                continue;
            }
            if (set.max_buffers_per_spectrum > 1) {
                cores[k]->combineResults(common_spec.data(), common_pcal.data());
                if (++combined == set.max_buffers_per_spectrum) {
                    for (int i = 0; i < set.num_sinks; i++) {
                        sink_ok &= (i < nsrc ? auto_sink(i) : snk[2]).write(common_spec[i]);
                        cores[0]->resetBuffer(common_spec[i]);
                    }
                    if (set.extract_PCal)
                        for (int s = 0; s < nsrc; s++) {
                            sink_ok &= pcal_sink(s).write(common_pcal[s]);
                            cores[0]->resetBuffer(common_pcal[s]);
                        }
                    total++;
                    combined = 0;
                }
            } else {
                for (int s = 0; s < nsrc; s++) sink_ok &= auto_sink(s).write(out[k][s]);
                for (int x = 0; x < set.num_xpols; x++) sink_ok &= snk[2].write(xpol[k][x]);
                if (set.extract_PCal)
                    for (int s = 0; s < nsrc; s++) {
                        sink_ok &= pcal_sink(s).write(pcal[k][s]);
                        cores[0]->resetBuffer(pcal[k][s]);
                    }
                total += n;
            }
        }
        db = (db + 1) % 2;
        bool more = false;
        for (int s = 0; s < nsrc; s++) more |= raw[0][db][s]->getLength() > 0;
        if (!more || rc) break;
    }
    for (auto& core : cores) core->finalize();
    for (int i = 0; i < 5; i++) sink_bytes[i] = snk[i].used;
    if (spectra_written) *spectra_written = total;
    if (rc) return rc;
    if (!sink_ok) return set_err("taskcore: a sink ran out of room");
    return 0;
}
