// TaskCoreCUDA: the swspectrometer computing core on the GPU (declared in
// include/TaskCoreCUDA.h).
//
// TaskCoreIPP (spectrometer/src/IA-32/TaskCoreIPP.cpp) is the core this
// replaces; the behaviour kept from it, by method:
// * prepare (:70-160): settings are read once; a worker thread per core waits
//   for work, as taskcoreipp_worker (:239-265) does.
// * run (:170-181) hands the buffers to the worker and returns 0; join
//   (:188-198) waits and returns the number of complete spectra.
// * doMaths (:394-513): the own output buffers are cleared, then as many
//   whole spectra as the shortest source holds are computed -- each spectrum
//   core_overlapped_ffts windowed FFTs with hop N/overlap over
//   core_averaged_ffts * N samples, |X|^2 with DC and Nyquist from the real
//   parts, the cross product of the two sources, the phase-cal fold of
//   every overlap-th FFT (the FFT count runs on across sources and spectra),
//   scaled by 1/core_overlapped_ffts -- and the buffer lengths are set to
//   the spectra written.  A trailing part of a buffer that holds no whole
//   spectrum (the reference writes it unscaled as a "partial" spectrum and
//   logs that this should only happen at an early end of file) is dropped
//   with a message on stderr.
// * combineResults (:311-349): the first spectrum of each source, the cross
//   spectrum and the phase-cal bins are added into the dispatcher's buffers
//   -- here on the GPU (cellspe_accumulate_f32) -- the lengths set as the
//   reference sets them (the cross spectrum's to fft_ssb_points floats, as
//   :334 does), and the core's own results cleared.
// * resetBuffer (:303-306): the buffer's allocated bytes set to 0.0 floats.
// The unpackers TaskCoreIPP would pick (DataUnpackerFactory.h:38-103) map to
// the engine's level tables and channel order: TwoBitUnpacker
// (DataUnpackers.cpp:174-232; map {+1, -1, +H, -H}, channel c in byte c/4 at
// bits 2(c%4), or mirrored when channelorder_increasing is false),
// Mark5BUnpacker (:305-376, the same map, increasing order) and
// Mk5BUnpacker (:597-680, mark5access levels {-H, +1, -1, +H}).
#include "TaskCoreCUDA.h"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <iostream>
#include <vector>

#include "Buffer.h"
#include "cellspe_gpu.h"

namespace {

// the 2-bit level table each of TaskCoreIPP's unpackers applies
int levels_for(InputFormat f, int* levels)
{
    switch (f) {
        case RawSigned:
        case RawUnsigned:
        case Mark5B: *levels = CELLSPE_LEVELS_TWOBIT; return 0;
        case Mk5B: *levels = CELLSPE_LEVELS_MARK5B; return 0;
        default: return -1;
    }
}

}  // namespace

TaskCoreCUDA::TaskCoreCUDA(int rank) : TaskCore(rank), rank_(rank) {}

TaskCoreCUDA::TaskCoreCUDA() : TaskCore(), rank_(0) {}

TaskCoreCUDA::~TaskCoreCUDA()
{
    finalize();
}

int TaskCoreCUDA::fail(const char* msg)
{
    std::snprintf(error_, sizeof error_, "TaskCoreCUDA core %d: %s", rank_, msg);
    std::cerr << error_ << std::endl;
    return -1;
}

void TaskCoreCUDA::prepare(swspect_settings_t* settings)
{
    cfg_ = settings;
    ok_ = false;
    error_[0] = 0;
    if (!cfg_) {
        fail("prepare: no settings");
        return;
    }
    const int N = (int)cfg_->fft_points, ov = cfg_->fft_overlap_factor;
    K_ = cfg_->core_averaged_ffts;
    nsub_ = cfg_->source_channels;
    nsrc_ = cfg_->num_sources;
    nxpol_ = cfg_->num_xpols;
    if (cfg_->bits_per_sample != 2) {
        fail("prepare: only 2-bit samples are supported");
    } else if (!(nsub_ == 4 || nsub_ == 8 || nsub_ == 16)) {
        fail("prepare: source_channels must be 4, 8 or 16");
    } else if (levels_for(cfg_->sourceformat, &levels_)) {
        fail("prepare: source format has no 2-bit unpacker here (RawSigned, RawUnsigned, Mark5B, Mk5B)");
    } else if (nsrc_ < 1 || nsrc_ > 2 || nxpol_ < 0 || nxpol_ > 1 || (nxpol_ == 1 && nsrc_ != 2)) {
        fail("prepare: one or two sources and at most one cross product");
    } else if (K_ < 1 || ov < 1 || cfg_->core_overlapped_ffts != ov * K_ - (ov - 1)) {
        fail("prepare: core_overlapped_ffts must be overlap * core_averaged_ffts - (overlap - 1)");
    } else if (cfg_->fft_ssb_points != N / 2 + 1) {
        fail("prepare: fft_ssb_points must be fft_points/2 + 1");
    } else if (cfg_->wf_type < None || cfg_->wf_type > Blackman) {
        fail("prepare: unknown window function");
    } else {
        const int ch[2] = {cfg_->use_channel_file1, cfg_->use_channel_file2};
        ok_ = true;
        for (int s = 0; s < nsrc_; s++) {
            if (ch[s] < 0 || ch[s] >= nsub_) {
                ok_ = false;
                fail("prepare: use_channel_file out of range");
                break;
            }
            // TwoBitUnpacker with decreasing order: channel c sits where the
            // increasing order keeps channel source_channels - 1 - c
            const bool mirrored = (cfg_->sourceformat == RawSigned || cfg_->sourceformat == RawUnsigned) &&
                                  !cfg_->channelorder_increasing;
            chan_[s] = mirrored ? nsub_ - 1 - ch[s] : ch[s];
        }
    }
    std::lock_guard<std::mutex> lk(mu_);
    if (!thread_.joinable()) {
        stage_ = IDLE;
        thread_ = std::thread(&TaskCoreCUDA::worker, this);
    }
}

int TaskCoreCUDA::run(Buffer** inbuf, Buffer** outbuf, Buffer** xpolbuf, Buffer** pcalbuf)
{
    std::lock_guard<std::mutex> lk(mu_);
    in_ = inbuf;
    out_ = outbuf;
    xpol_ = xpolbuf;
    pcal_ = pcalbuf;
    if (!thread_.joinable()) {        // run() without prepare()
        result_ = fail("run: prepare() was not called");
        stage_ = DONE;
        return 0;
    }
    stage_ = QUEUED;
    cv_.notify_all();
    return 0;
}

int TaskCoreCUDA::join()
{
    std::unique_lock<std::mutex> lk(mu_);
    cv_.wait(lk, [&] { return stage_ == DONE || stage_ == IDLE; });
    if (stage_ == IDLE) return -1;   // nothing was started
    stage_ = IDLE;
    return result_;
}

void TaskCoreCUDA::worker()
{
    std::unique_lock<std::mutex> lk(mu_);
    for (;;) {
        cv_.wait(lk, [&] { return stage_ == QUEUED || stage_ == QUIT; });
        if (stage_ == QUIT) return;
        lk.unlock();
        const int r = compute();
        lk.lock();
        result_ = r;
        if (stage_ != QUIT) stage_ = DONE;
        cv_.notify_all();
    }
}

bool TaskCoreCUDA::grow(void** p, size_t* cap, size_t bytes)
{
    if (*cap >= bytes && *p) return true;
    if (*p) cellspe_device_free(*p);
    *p = cellspe_device_alloc(bytes);
    *cap = *p ? bytes : 0;
    return *p != nullptr;
}

void TaskCoreCUDA::resetBuffer(Buffer* buf)
{
    if (buf && buf->getData()) std::memset(buf->getData(), 0, buf->getAllocated() / sizeof(float) * sizeof(float));
}

int TaskCoreCUDA::compute()
{
    if (!ok_) return error_[0] ? -1 : fail("run: settings were not accepted");
    if (!in_ || !out_ || (nxpol_ && !xpol_) || (cfg_->extract_PCal && !pcal_)) return fail("run: null buffer array");
    const long long N = (long long)cfg_->fft_points, nb = N / 2 + 1;
    const long long bpt = nsub_ / 4;                         // raw bytes per sample time
    const long long spec_bytes = (long long)K_ * N * bpt;    // raw bytes of one (sub-)spectrum
    const bool pcal = cfg_->extract_PCal && cfg_->pcal_tonebins > 0;
    const long long T = pcal ? cfg_->pcal_tonebins : 0;

    // the own results are cleared first (reset_spectrum, TaskCoreIPP.cpp:274-293)
    have_results_ = false;
    for (int s = 0; s < nsrc_; s++) resetBuffer(out_[s]);
    for (int x = 0; x < nxpol_; x++) resetBuffer(xpol_[x]);
    if (pcal)
        for (int s = 0; s < nsrc_; s++) resetBuffer(pcal_[s]);

    long long len = (long long)in_[0]->getLength();
    for (int s = 1; s < nsrc_; s++) len = std::min(len, (long long)in_[s]->getLength());
    const long long nspec = len / spec_bytes;
    if (len - nspec * spec_bytes >= N * bpt)
        std::cerr << "TaskCoreCUDA core " << rank_ << ": " << (len - nspec * spec_bytes) / (N * bpt)
                  << " FFT lengths of raw data after the last whole spectrum are not used" << std::endl;
    nspec_ = (int)nspec;
    auto set_lengths = [&](long long n) {
        for (int s = 0; s < nsrc_; s++) out_[s]->setLength(cfg_->fft_bytes_ssb * n);
        for (int x = 0; x < nxpol_; x++) xpol_[x]->setLength(cfg_->fft_bytes_xpol * n);
        if (pcal)
            for (int s = 0; s < nsrc_; s++) pcal_[s]->setLength(cfg_->pcal_result_bytes * n);
    };
    if (nspec == 0) {
        set_lengths(0);
        return 0;
    }
    for (int s = 0; s < nsrc_; s++)
        if ((long long)out_[s]->getAllocated() < nspec * nb * 4 ||
            (pcal && (long long)pcal_[s]->getAllocated() < nspec * T * 8))
            return fail("run: output buffer too small for the spectra of the raw buffer");
    for (int x = 0; x < nxpol_; x++)
        if ((long long)xpol_[x]->getAllocated() < nspec * nb * 8) return fail("run: cross-spectrum buffer too small");

    const long long raw_bytes = nspec * spec_bytes;
    for (int s = 0; s < nsrc_; s++) {
        if (!grow(&d_raw_[s], &raw_cap_[s], (size_t)raw_bytes)) return fail("run: device memory for raw data");
        if (cellspe_memcpy(d_raw_[s], in_[s]->getData(), (size_t)raw_bytes, 1))
            return fail(cellspe_last_error());
    }
    cellspe_spec_params p;
    std::memset(&p, 0, sizeof p);
    p.fft_points = (int)N;
    p.overlap = cfg_->fft_overlap_factor;
    p.window = (int)cfg_->wf_type;
    p.ffts_per_spectrum = K_;
    p.n_spectra = (int)nspec;
    p.n_subbands = nsub_;
    p.input_layout = CELLSPE_SPEC_INTERLEAVED;
    p.levels = levels_;
    p.raw_bytes = raw_bytes;
    p.pcal_tonebins = (int)T;
    p.pcal_rotatorlen = pcal ? cfg_->pcal_rotatorlen : 0;
    p.pcal_ntones = 0;
    p.pcal_offset_hz = cfg_->pcaloffsethz;
    p.sample_rate_hz = cfg_->samplingfreq;
    p.memory = CELLSPE_MEM_DEVICE;

    if (nsrc_ == 1) {
        // every subband is computed; the source's channel is read back
        if (!grow(&d_power_, &power_cap_, (size_t)(nsub_ * nspec * nb * 4)) ||
            (pcal && !grow(&d_pcal_, &pcal_cap_, (size_t)(nsub_ * nspec * T * 8))))
            return fail("run: device memory for spectra");
        if (cellspe_spectrometer(&p, d_raw_[0], (float*)d_power_, pcal ? d_pcal_ : nullptr, nullptr))
            return fail(cellspe_last_error());
        own_power_[0] = (float*)d_power_ + (size_t)chan_[0] * nspec * nb;
        own_pcal_[0] = pcal ? (float*)d_pcal_ + (size_t)chan_[0] * nspec * T * 2 : nullptr;
        own_xpol_ = nullptr;
    } else {
        if (!grow(&d_power_, &power_cap_, (size_t)(2 * nspec * nb * 4)) ||
            !grow(&d_xpol_, &xpol_cap_, (size_t)(nspec * nb * 8)) ||
            (pcal && !grow(&d_pcal_, &pcal_cap_, (size_t)(2 * nspec * T * 8))))
            return fail("run: device memory for spectra");
        if (cellspe_spectrometer_xpol(&p, d_raw_[0], d_raw_[1], chan_[0], chan_[1], (float*)d_power_, d_xpol_,
                                      pcal ? d_pcal_ : nullptr))
            return fail(cellspe_last_error());
        for (int s = 0; s < 2; s++) {
            own_power_[s] = (float*)d_power_ + (size_t)s * nspec * nb;
            own_pcal_[s] = pcal ? (float*)d_pcal_ + (size_t)s * nspec * T * 2 : nullptr;
        }
        own_xpol_ = (float*)d_xpol_;
    }
    for (int s = 0; s < nsrc_; s++) {
        if (cellspe_memcpy(out_[s]->getData(), own_power_[s], (size_t)(nspec * nb * 4), 2)) return fail(cellspe_last_error());
        if (pcal && cellspe_memcpy(pcal_[s]->getData(), own_pcal_[s], (size_t)(nspec * T * 8), 2))
            return fail(cellspe_last_error());
    }
    for (int x = 0; x < nxpol_; x++)
        if (cellspe_memcpy(xpol_[x]->getData(), own_xpol_, (size_t)(nspec * nb * 8), 2)) return fail(cellspe_last_error());
    set_lengths(nspec);
    have_results_ = true;
    return (int)nspec;
}

int TaskCoreCUDA::combineResults(Buffer** outbuf, Buffer** pcalbuf)
{
    if (!outbuf || !pcalbuf || !out_ || !pcal_) {
        std::cerr << "TaskCoreCUDA combine : null buffer(s)!" << std::endl;
        return 0;
    }
    const long long nb = cfg_->fft_ssb_points;
    const bool pcal = cfg_->extract_PCal && cfg_->pcal_tonebins > 0;
    const long long T = pcal ? cfg_->pcal_tonebins : 0;
    // dst (host, n floats) += src (device), summed on the device
    auto add = [&](Buffer* dst, const float* src, long long n) -> int {
        if (!dst || (long long)dst->getAllocated() < n * 4) return fail("combine: common buffer too small");
        if (!grow(&d_acc_, &acc_cap_, (size_t)n * 4)) return fail("combine: device memory");
        if (cellspe_memcpy(d_acc_, dst->getData(), (size_t)n * 4, 1) ||
            cellspe_accumulate_f32((float*)d_acc_, src, n, CELLSPE_MEM_DEVICE) ||
            cellspe_memcpy(dst->getData(), d_acc_, (size_t)n * 4, 2))
            return fail(cellspe_last_error());
        return 0;
    };
    if (have_results_) {
        for (int s = 0; s < nsrc_; s++) add(outbuf[s], own_power_[s], nb);
        for (int x = 0; x < nxpol_; x++) add(outbuf[x + nsrc_], own_xpol_, 2 * nb);
        if (pcal)
            for (int s = 0; s < nsrc_; s++) add(pcalbuf[s], own_pcal_[s], 2 * T);
    }
    for (int s = 0; s < nsrc_; s++) outbuf[s]->setLength(sizeof(float) * nb);
    for (int x = 0; x < nxpol_; x++) outbuf[x + nsrc_]->setLength(sizeof(float) * nb);
    if (pcal)
        for (int s = 0; s < nsrc_; s++) pcalbuf[s]->setLength(sizeof(float) * 2 * T);
    // the own results are cleared (reset_spectrum)
    have_results_ = false;
    for (int s = 0; s < nsrc_; s++) resetBuffer(out_[s]);
    for (int x = 0; x < nxpol_; x++) resetBuffer(xpol_[x]);
    if (pcal)
        for (int s = 0; s < nsrc_; s++) resetBuffer(pcal_[s]);
    return 0;
}

void TaskCoreCUDA::releaseDevice()
{
    for (int s = 0; s < 2; s++) {
        if (d_raw_[s]) cellspe_device_free(d_raw_[s]);
        d_raw_[s] = nullptr;
        raw_cap_[s] = 0;
    }
    void** bufs[] = {&d_power_, &d_xpol_, &d_pcal_, &d_acc_};
    for (void** b : bufs) {
        if (*b) cellspe_device_free(*b);
        *b = nullptr;
    }
    power_cap_ = xpol_cap_ = pcal_cap_ = acc_cap_ = 0;
    have_results_ = false;
}

int TaskCoreCUDA::finalize()
{
    {
        std::lock_guard<std::mutex> lk(mu_);
        if (!thread_.joinable()) {
            releaseDevice();
            return 0;
        }
        stage_ = QUIT;
        cv_.notify_all();
    }
    thread_.join();
    releaseDevice();
    return 0;
}
