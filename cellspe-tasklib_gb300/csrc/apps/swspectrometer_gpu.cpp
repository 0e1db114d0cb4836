// swspectrometer_gpu -- the spectrometer entry point on the GB300 engine.
//
// Usage: swspectrometer_gpu <ini file> <input file 1> [<input file 2>]
//
// Mirrors the reference's swspectrometer (spectrometer/src/swspectrometer.cpp):
// the [Spectrometer] section of the INI file is read with the same keys and
// defaults (:67-146), the same settings are derived (:161-232), and one power
// spectrum per integration period is written per input file to
// <BaseFilename>_swspec.bin (N/2+1 float32 per spectrum, FileSink.cpp:52-103),
// plus the folded phase-cal bins to <BaseFilename>_pcal.bin when ExtractPCal
// is set.  The arithmetic runs in cellspe_spectrometer (TaskCoreIPP::doMaths
// on the GPU) for all subbands of the input at once; the file keeps the
// subband named by UseFile1Channel.  With two input files (two sources) the
// spectra come from cellspe_spectrometer_xpol: the second source's auto
// spectra go to <BaseFilename>_file2_swspec.bin and the cross-polarisation
// spectrum (N/2+1 complex64 per spectrum) to <BaseFilename>_xpol_swspec.bin.
//
// Input: 2-bit samples (BitsPerSample = 2), SourceChannels channels
// interleaved per sample time.  SourceFormat selects the framing as
// FileSource::open does (FileSource.cpp:40-62): "Mark5B" is a framed Mark5B
// recording (16-byte headers, 10000-byte payloads, first frame searched for),
// "VDIF" a framed VDIF recording (frames from byte 0, frame length from the
// first header; Mbps = 2 x BandwidthHz x 2 bits x SourceChannels); headers are
// stripped and invalid or fill-pattern data blanked on the GPU, as mark5access
// decodes them (FileSource passes fill bytes through as samples, and the
// reference has no VDIF unpacker).  A framed file is read whole and its
// spectra computed in one call, so the phase-cal FFT count runs on across
// them as in a reference core buffer holding the whole file.  Any other
// SourceFormat is headerless payload (Mark5B payload order, or the TwoBit
// order with ChannelOrderIncreasing; names starting with "Mark5B" use the
// mark5access level table, anything else the TwoBitUnpacker table), read one
// integration period per call.
// Differences from the reference: a zero PCalOffsetHz uses the comb period as
// rotator length (the reference divides by zero in Helpers::gcd), and the
// data of one integration period are read per GPU call instead of buffers
// sized by MaxSourceBufferMB.  The phase-cal windows therefore match a
// reference run whose core buffers hold one spectrum each: the reference's
// FFT count runs on across the spectra of one buffer, so with several spectra
// per buffer and FFToverlapFactor > 1 its later spectra fold other windows.
#include "../../../include/cellspe_gpu.h"

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <string>
#include <vector>

namespace {

std::string lower(std::string s)
{
    for (auto& c : s) c = (char)tolower((unsigned char)c);
    return s;
}

std::string trim(const std::string& s)
{
    size_t b = s.find_first_not_of(" \t\r\n"), e = s.find_last_not_of(" \t\r\n");
    return b == std::string::npos ? std::string() : s.substr(b, e - b + 1);
}

// Minimal INI reader: [section] headers, key = value lines, ';' or '#'
// comments; keys compared case-insensitively (IniParser.h:39-99).
std::map<std::string, std::string> read_section(const char* path, const std::string& section)
{
    std::map<std::string, std::string> kv;
    std::ifstream f(path);
    std::string line, cur;
    while (std::getline(f, line)) {
        line = trim(line);
        if (line.empty() || line[0] == ';' || line[0] == '#') continue;
        if (line[0] == '[') {
            cur = lower(trim(line.substr(1, line.find(']') - 1)));
            continue;
        }
        size_t eq = line.find('=');
        if (eq == std::string::npos || cur != lower(section)) continue;
        std::string v = trim(line.substr(eq + 1));
        if (v.size() >= 2 && v.front() == '"' && v.back() == '"') v = v.substr(1, v.size() - 2);
        kv[lower(trim(line.substr(0, eq)))] = v;
    }
    return kv;
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

struct Settings {
    int fft_points = 320000, overlap = 2, window = 2, channels = 1, bits = 8;
    int use_ch[2] = {1, 1};
    double integ_s = 20.0, fs = 16e6, pcal_offset = 10e3, pcal_spacing = 1e6;
    bool pcal = false, ascii = false, mark5b = false;
    std::string base = "ProjDate_StationID_Instrument_ScanNo_%fftpoints%_%integrtime%_%channel%";
    std::string format = "RawSigned";
};

std::string fill_pattern(std::string pat, const Settings& s, int ch)
{
    auto rep = [&](const std::string& key, const std::string& val) {
        size_t i;
        while ((i = pat.find(key)) != std::string::npos) pat.replace(i, key.size(), val);
    };
    rep("%fftpoints%", std::to_string(s.fft_points));
    rep("%integrtime%", std::to_string((int)s.integ_s));
    rep("%channel%", std::to_string(ch));
    return pat;
}

}  // namespace

int main(int argc, char** argv)
{
    if (argc < 3 || argc > 4) {
        std::cerr << "Usage: " << argv[0] << " <inifile> <datafile1> [<datafile2>]\n";
        return argc == 1 ? 0 : -1;
    }
    auto kv = read_section(argv[1], "Spectrometer");
    if (kv.empty()) {
        std::cerr << "Error: INI could not be read or it is missing the [Spectrometer] section\n";
        return -1;
    }
    Settings s;
    auto geti = [&](const char* k, int& v) { if (kv.count(k)) v = atoi(kv[k].c_str()); };
    auto getd = [&](const char* k, double& v) { if (kv.count(k)) v = atof(kv[k].c_str()); };
    auto getb = [&](const char* k, bool& v) {
        if (kv.count(k)) { std::string x = lower(kv[k]); v = (x == "1" || x == "true" || x == "yes"); }
    };
    geti("fftpoints", s.fft_points);
    getd("fftintegrationtimesec", s.integ_s);
    geti("fftoverlapfactor", s.overlap);
    if (kv.count("windowtype")) {
        std::string w = lower(kv["windowtype"]);
        s.window = (w == "none") ? 0 : (w == "cosine") ? 1 : (w == "cosine2") ? 2 : -1;
        if (s.window < 0) { std::cerr << "Error: window " << kv["windowtype"] << " is not available on the GPU engine\n"; return -1; }
    }
    if (kv.count("bandwidthhz")) s.fs = 2.0 * atof(kv["bandwidthhz"].c_str());      // fs = 2 BW
    getd("pcaloffsethz", s.pcal_offset);
    if (kv.count("sourceformat")) s.format = kv["sourceformat"];
    geti("bitspersample", s.bits);
    geti("sourcechannels", s.channels);
    geti("usefile1channel", s.use_ch[0]);
    geti("usefile2channel", s.use_ch[1]);
    getb("extractpcal", s.pcal);
    s.ascii = kv.count("sinkformat") && lower(kv["sinkformat"]) == "ascii";
    if (!kv.count("basefilename1")) {
        std::cerr << "Error: BaseFilename1 setting is missing from the INI file!\n";
        return -1;
    }
    s.base = kv["basefilename1"];
    s.mark5b = lower(s.format).rfind("mark5b", 0) == 0;
    if (s.bits != 2) { std::cerr << "Error: the GPU engine reads 2-bit data (BitsPerSample = 2)\n"; return -1; }
    for (int f = 0; f < 2; f++)
        if (s.use_ch[f] < 1 || s.use_ch[f] > s.channels) {
            std::cerr << "Error: UseFile" << (f + 1) << "Channel setting " << s.use_ch[f] << " is an invalid channel number\n";
            return -1;
        }

    // derived settings (swspectrometer.cpp:161-232)
    const long long N = s.fft_points;
    const long long K = (long long)(s.fs * s.integ_s) / N;             // averaged FFTs per spectrum
    const int tonebins = s.pcal ? (int)(s.fs / s.pcal_spacing) : 0;
    const long long off = (long long)s.pcal_offset;
    const int rotlen = s.pcal ? (off == 0 ? tonebins : (int)((long long)s.fs / gcd_ll((long long)s.fs, off))) : 0;
    const int ntones = s.pcal ? (int)(s.fs / 2 / s.pcal_spacing) : 0;
    const long long bytes_per_spec = K * N * s.channels / 4;
    if (K < 1) { std::cerr << "Error: integration shorter than one FFT\n"; return -1; }

    cellspe_spec_params p;
    std::memset(&p, 0, sizeof p);
    p.fft_points = (int)N; p.overlap = s.overlap; p.window = s.window; p.ffts_per_spectrum = (int)K;
    p.n_spectra = 1; p.n_subbands = s.channels; p.input_layout = CELLSPE_SPEC_INTERLEAVED;
    p.levels = s.mark5b ? CELLSPE_LEVELS_MARK5B : CELLSPE_LEVELS_TWOBIT;
    p.raw_bytes = bytes_per_spec; p.pcal_tonebins = tonebins; p.pcal_rotatorlen = rotlen;
    p.pcal_ntones = 0; p.pcal_offset_hz = s.pcal_offset; p.sample_rate_hz = s.fs; p.memory = CELLSPE_MEM_HOST;

    if (argc == 4) {
        // two sources: auto spectra of both plus the cross spectrum
        // (TaskCoreIPP::doMaths with num_sources = 2, num_xpols = 1;
        // swspectrometer.cpp:247-254, 341-358 name the outputs)
        std::ifstream in0(argv[2], std::ios::binary), in1(argv[3], std::ios::binary);
        if (!in0 || !in1) { std::cerr << "Error: cannot open the input files\n"; return -1; }
        const std::string base1 = fill_pattern(s.base, s, s.use_ch[0]);
        const std::string base2 = fill_pattern(s.base + "_file2", s, s.use_ch[1]);
        std::ofstream out0(base1 + "_swspec.bin", std::ios::binary), out1(base2 + "_swspec.bin", std::ios::binary);
        std::ofstream outx(base1 + "_xpol_swspec.bin", std::ios::binary);
        std::ofstream pout0, pout1;
        if (s.pcal) { pout0.open(base1 + "_pcal.bin", std::ios::binary); pout1.open(base2 + "_pcal.bin", std::ios::binary); }
        void* raw0 = cellspe_host_alloc((size_t)bytes_per_spec);
        void* raw1 = cellspe_host_alloc((size_t)bytes_per_spec);
        if (!raw0 || !raw1) { std::cerr << "Error: " << cellspe_last_error() << "\n"; return -1; }
        std::vector<float> power((size_t)2 * (N / 2 + 1)), xpol((size_t)2 * (N / 2 + 1));
        std::vector<float> bins((size_t)2 * std::max(tonebins, 1) * 2);
        long long nspec = 0;
        int status = 0;
        while (in0.read((char*)raw0, bytes_per_spec) && in0.gcount() == bytes_per_spec &&
               in1.read((char*)raw1, bytes_per_spec) && in1.gcount() == bytes_per_spec) {
            int rc = cellspe_spectrometer_xpol(&p, raw0, raw1, s.use_ch[0] - 1, s.use_ch[1] - 1, power.data(),
                                               xpol.data(), s.pcal ? bins.data() : nullptr);
            if (rc) { std::cerr << "Error: " << cellspe_last_error() << "\n"; status = -1; break; }
            out0.write((const char*)power.data(), sizeof(float) * (N / 2 + 1));
            out1.write((const char*)(power.data() + (N / 2 + 1)), sizeof(float) * (N / 2 + 1));
            outx.write((const char*)xpol.data(), sizeof(float) * 2 * (N / 2 + 1));
            if (s.pcal) {
                pout0.write((const char*)bins.data(), sizeof(float) * 2 * tonebins);
                pout1.write((const char*)(bins.data() + 2 * tonebins), sizeof(float) * 2 * tonebins);
            }
            nspec++;
        }
        std::cerr << nspec << " spectra of " << N << " points from two sources (channels " << s.use_ch[0] << ", "
                  << s.use_ch[1] << ") -> " << base1 << "_xpol_swspec.bin\n";
        cellspe_host_free(raw0);
        cellspe_host_free(raw1);
        return status;
    }

    const std::string fmt_l = lower(s.format);
    if (fmt_l == "mark5b" || fmt_l == "vdif") {
        // framed recordings: whole files, headers stripped on the GPU
        const bool vdif = fmt_l == "vdif";
        const int nsrc = argc - 2;
        std::vector<void*> bufs(nsrc, nullptr);
        long long nspec = -1, bytes = 0;
        for (int f = 0; f < nsrc; f++) {
            std::ifstream in(argv[2 + f], std::ios::binary | std::ios::ate);
            if (!in) { std::cerr << "Error: cannot open " << argv[2 + f] << "\n"; return -1; }
            const long long sz = (long long)in.tellg();
            in.seekg(0);
            if (f == 0) bytes = sz;
            if (sz != bytes) { std::cerr << "Error: the two framed inputs differ in size\n"; return -1; }
            bufs[f] = cellspe_host_alloc((size_t)std::max(sz, 1LL));
            if (!bufs[f] || !in.read((char*)bufs[f], sz)) { std::cerr << "Error: cannot read " << argv[2 + f] << "\n"; return -1; }
            long long samples = 0;
            if (vdif) {
                cellspe_vdif_info info;
                const int mbps = (int)llround(s.fs * 2.0 * s.channels / 1e6);
                if (cellspe_vdif_deframe(bufs[f], sz, s.channels, mbps, 0, nullptr, nullptr, CELLSPE_MEM_HOST, &info)) {
                    std::cerr << "Error: " << cellspe_last_error() << "\n";
                    return -1;
                }
                samples = info.frames * ((long long)(info.frame_bytes - info.header_bytes) * 4 / s.channels);
            } else {
                cellspe_mark5b_info info;
                if (cellspe_mark5b_deframe(bufs[f], sz, s.channels, 0, nullptr, nullptr, CELLSPE_MEM_HOST, &info)) {
                    std::cerr << "Error: " << cellspe_last_error() << "\n";
                    return -1;
                }
                samples = info.frames * (10000LL * 4 / s.channels);
            }
            const long long n = samples / (K * N);
            nspec = nspec < 0 ? n : std::min(nspec, n);
        }
        if (nspec < 1) { std::cerr << "Error: the framed input holds less than one integration period\n"; return -1; }
        p.input_layout = vdif ? CELLSPE_SPEC_VDIF_FRAMED : CELLSPE_SPEC_MARK5B_FRAMED;
        p.levels = vdif ? CELLSPE_LEVELS_VDIF : CELLSPE_LEVELS_MARK5B;
        p.raw_bytes = bytes;
        p.n_spectra = (int)nspec;
        const long long nb = N / 2 + 1;
        const std::string base1 = fill_pattern(s.base, s, s.use_ch[0]);
        int rc;
        if (nsrc == 2) {
            const std::string base2 = fill_pattern(s.base + "_file2", s, s.use_ch[1]);
            std::vector<float> power((size_t)2 * nspec * nb), xpol((size_t)2 * nspec * nb);
            std::vector<float> bins((size_t)2 * nspec * std::max(tonebins, 1) * 2);
            rc = cellspe_spectrometer_xpol(&p, bufs[0], bufs[1], s.use_ch[0] - 1, s.use_ch[1] - 1, power.data(),
                                           xpol.data(), s.pcal ? bins.data() : nullptr);
            if (!rc) {
                std::ofstream(base1 + "_swspec.bin", std::ios::binary).write((const char*)power.data(), sizeof(float) * nspec * nb);
                std::ofstream(base2 + "_swspec.bin", std::ios::binary)
                    .write((const char*)(power.data() + nspec * nb), sizeof(float) * nspec * nb);
                std::ofstream(base1 + "_xpol_swspec.bin", std::ios::binary)
                    .write((const char*)xpol.data(), sizeof(float) * 2 * nspec * nb);
                if (s.pcal) {
                    std::ofstream(base1 + "_pcal.bin", std::ios::binary).write((const char*)bins.data(), sizeof(float) * 2 * nspec * tonebins);
                    std::ofstream(base2 + "_pcal.bin", std::ios::binary)
                        .write((const char*)(bins.data() + 2 * nspec * tonebins), sizeof(float) * 2 * nspec * tonebins);
                }
            }
        } else {
            const int ch = s.use_ch[0];
            std::vector<float> power((size_t)s.channels * nspec * nb);
            std::vector<float> bins((size_t)s.channels * nspec * std::max(tonebins, 1) * 2);
            rc = cellspe_spectrometer(&p, bufs[0], power.data(), s.pcal ? bins.data() : nullptr, nullptr);
            if (!rc) {
                std::ofstream out(base1 + "_swspec.bin", s.ascii ? std::ios::out : std::ios::binary);
                for (long long sp = 0; sp < nspec; sp++) {
                    const float* spec = power.data() + ((size_t)(ch - 1) * nspec + sp) * nb;
                    if (s.ascii) {
                        out << "// --------------------- DATA SET TIMESTAMP xxxx ---------------------\n";
                        out << "// FFT bins 0.." << (N / 2) << " + Nyquist\n";
                        for (long long k = 0; k < nb; k++) out << spec[k] << "\n";
                    } else {
                        out.write((const char*)spec, sizeof(float) * nb);
                    }
                }
                if (s.pcal)
                    std::ofstream(base1 + "_pcal.bin", std::ios::binary)
                        .write((const char*)(bins.data() + (size_t)(ch - 1) * nspec * tonebins * 2),
                               sizeof(float) * 2 * nspec * tonebins);
            }
        }
        for (void* b : bufs) cellspe_host_free(b);
        if (rc) { std::cerr << "Error: " << cellspe_last_error() << "\n"; return -1; }
        std::cerr << nspec << " spectra of " << N << " points from framed " << s.format << " input -> " << base1
                  << "_swspec.bin\n";
        return 0;
    }

    int status = 0;
    for (int f = 0; f < argc - 2; f++) {
        std::ifstream in(argv[2 + f], std::ios::binary);
        if (!in) { std::cerr << "Error: cannot open " << argv[2 + f] << "\n"; return -1; }
        const int ch = s.use_ch[f];
        const std::string base = fill_pattern(f == 0 ? s.base : s.base + "_file2", s, ch);
        std::ofstream out(base + "_swspec.bin", s.ascii ? std::ios::out : std::ios::binary);
        std::ofstream pout;
        if (s.pcal) pout.open(base + "_pcal.bin", std::ios::binary);
        void* raw = cellspe_host_alloc((size_t)bytes_per_spec);
        std::vector<float> power((size_t)s.channels * (N / 2 + 1));
        std::vector<float> bins((size_t)s.channels * std::max(tonebins, 1) * 2);
        if (!raw) { std::cerr << "Error: " << cellspe_last_error() << "\n"; return -1; }
        long long nspec = 0;
        while (in.read((char*)raw, bytes_per_spec) && in.gcount() == bytes_per_spec) {
            int rc = cellspe_spectrometer(&p, raw, power.data(), s.pcal ? bins.data() : nullptr, nullptr);
            if (rc) { std::cerr << "Error: " << cellspe_last_error() << "\n"; status = -1; break; }
            const float* spec = power.data() + (size_t)(ch - 1) * (N / 2 + 1);
            if (s.ascii) {
                out << "// --------------------- DATA SET TIMESTAMP xxxx ---------------------\n";
                out << "// FFT bins 0.." << (N / 2) << " + Nyquist\n";
                for (long long k = 0; k <= N / 2; k++) out << spec[k] << "\n";
            } else {
                out.write((const char*)spec, sizeof(float) * (N / 2 + 1));
            }
            if (s.pcal) pout.write((const char*)(bins.data() + (size_t)(ch - 1) * tonebins * 2), sizeof(float) * 2 * tonebins);
            nspec++;
        }
        std::cerr << argv[2 + f] << ": " << nspec << " spectra of " << N << " points, " << K
                  << " FFTs averaged (overlap " << s.overlap << "), channel " << ch << " -> " << base << "_swspec.bin\n";
        cellspe_host_free(raw);
        (void)ntones;
    }
    return status;
}
