// C-ABI runtime of the GB300 engine: the celldsp_* task runtime
// (cellspe-tasklib.cpp:110-412), the spe* DSP wrappers
// (cellspe-tasklib-dsp.cpp:94-359) and the direct cellspe_* entry points.
//
// An execution slot replaces an SPE.  Each slot owns a host worker thread (the
// SPU main loop of cellspe-tasklib.cpp:440-617: take a task, run it, write
// completed_flag and tick_count, follow next_task), a CUDA stream and a
// device workspace.  Task vectors are host pointers by default, staged
// through the workspace; CELLDSP_TASK_FLAG_DEVPTR marks device pointers.
#include "../../include/cellspe_gpu.h"
#include "kernels.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <deque>
#include <unordered_map>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <iostream>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

namespace {

thread_local std::string t_err;

int set_err(int code, const std::string& msg)
{
    t_err = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char* where)
{
    return set_err(CELLSPE_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

int map_rc(int rc, const char* where)
{
    if (rc == 0) return CELLSPE_OK;
    if (rc == CS_ERR_ARG) return set_err(CELLSPE_ERR_ARG, std::string(where) + ": invalid argument");
    if (rc == CS_ERR_UNSUPPORTED) return set_err(CELLSPE_ERR_UNSUPPORTED, std::string(where) + ": unsupported size or mode");
    return cuda_fail((cudaError_t)rc, where);
}

#define RT_TRY(expr, where)                   \
    do {                                      \
        int _rc = map_rc((int)(expr), where); \
        if (_rc) return _rc;                  \
    } while (0)

std::atomic<long long> g_budget{0};
std::atomic<int> g_inject_direct{0};

int ensure_device()
{
    static std::once_flag once;
    static cudaError_t init_err = cudaSuccess;
    std::call_once(once, [] {
        int n = 0;
        init_err = cudaGetDeviceCount(&n);
        if (init_err == cudaSuccess && n == 0) init_err = cudaErrorNoDevice;
        if (init_err == cudaSuccess) init_err = cudaSetDevice(0);
        if (init_err == cudaSuccess) init_err = cudaFree(nullptr);
    });
    if (init_err != cudaSuccess) return cuda_fail(init_err, "GPU initialisation");
    return cudaSetDevice(0) == cudaSuccess ? 0 : cuda_fail(cudaGetLastError(), "cudaSetDevice");
}

size_t align256(size_t n) { return (n + 255) & ~(size_t)255; }

// Device workspace: a bump arena over one or more blocks.  After a job that
// needed several blocks, reset() merges them into one, so steady-state jobs of
// the same size allocate nothing.
// Device scratch of one workspace: bump allocation in the newest block; a
// request that does not fit takes a new block of at least 64 MiB, and the
// next reset() merges the blocks into one as large as the last job needed.
// Blocks come from the stream-ordered allocator on the workspace's stream
// (cudaMallocAsync / cudaFreeAsync): cudaFree would wait for the whole
// device, which in the correlation service holds one job up behind every
// other job's kernels.
struct Arena {
    std::vector<std::pair<char*, size_t>> blocks;
    size_t used = 0;
    size_t total_taken = 0;
    cudaStream_t stream = nullptr;    // the stream the blocks are ordered on
    size_t capacity() const
    {
        size_t c = 0;
        for (auto& b : blocks) c += b.second;
        return c;
    }
    void* take(size_t n, cudaError_t* err)
    {
        n = align256(std::max<size_t>(n, 1));
        total_taken += n;
        if (blocks.empty() || used + n > blocks.back().second) {
            char* p = nullptr;
            size_t sz = std::max(n, (size_t)64 << 20);
            cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&p), sz, stream);
            if (e != cudaSuccess) {
                *err = e;
                return nullptr;
            }
            blocks.push_back({p, sz});
            used = 0;
        }
        void* r = blocks.back().first + used;
        used += n;
        return r;
    }
    // the blocks' last users have finished (stream synchronised)
    void reset()
    {
        if (blocks.size() > 1) {
            size_t want = std::max(total_taken, capacity());
            for (auto& b : blocks) cudaFreeAsync(b.first, stream);
            blocks.clear();
            char* p = nullptr;
            if (cudaMallocAsync(reinterpret_cast<void**>(&p), want, stream) == cudaSuccess) blocks.push_back({p, want});
            else cudaGetLastError();
        }
        rewind();
    }
    // start the next job in the same blocks (no allocator calls: safe while
    // a CUDA graph is being captured)
    void rewind()
    {
        used = 0;
        total_taken = 0;
    }
    void release()
    {
        for (auto& b : blocks) cudaFreeAsync(b.first, stream);
        blocks.clear();
        used = total_taken = 0;
    }
};

// Host-buffer FX jobs move their input in PIPE_IN blocks of inputs and their
// visibilities in PIPE_OUT blocks of channels: more input blocks shorten the
// wait for the first one; output blocks stay large enough to fill the GPU.
constexpr int PIPE_IN = 16, PIPE_OUT = 8;

// Input-copy order shared by the workers of one service: a host-buffer job's
// input copies start after the previous job's input copies have finished
// (a device-side wait on `in_done`), so two jobs in flight do not copy and
// compute in lockstep (each at half speed) but one's input moves while the
// other computes.
struct CopyChain {
    std::mutex mu;
    cudaEvent_t in_done = nullptr;
    bool valid = false;
};

struct Workspace {
    CopyChain* chain = nullptr;       // set by the service for its workers
    cudaStream_t stream = nullptr;
    cudaStream_t copy = nullptr;      // host <-> device copies overlapping the kernels
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaEvent_t sev[5] = {};          // stage boundaries of the last FX job
    cudaEvent_t cev[PIPE_IN + PIPE_OUT + 2] = {};   // copy / compute hand-offs
    cudaEvent_t ev_legacy = nullptr;  // ordering after the legacy default stream
    Arena arena;
    bool own_stream = true;
    struct Out { void* host; const void* dev; size_t bytes; };
    std::vector<Out> outs;
    int init()
    {
        if (stream) return 0;
        int rc = ensure_device();
        if (rc) return rc;
        cudaError_t e = cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&copy, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreate(&ev0);
        if (e == cudaSuccess) e = cudaEventCreate(&ev1);
        for (auto& ev : sev)
            if (e == cudaSuccess) e = cudaEventCreate(&ev);
        for (auto& ev : cev)
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev_legacy, cudaEventDisableTiming);
        return e == cudaSuccess ? 0 : cuda_fail(e, "stream setup");
    }
    // The library's streams are non-blocking, so a call that reads device
    // buffers first waits (on the device, not the host) for everything issued
    // so far to the legacy default stream -- which itself waits for all
    // blocking streams -- so buffers that the caller's earlier work fills there
    // are complete.  Work on the caller's own non-blocking streams is the
    // caller's to synchronise.
    int after_legacy_stream()
    {
        cudaError_t e = cudaEventRecord(ev_legacy, cudaStreamLegacy);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(stream, ev_legacy, 0);
        return e == cudaSuccess ? 0 : cuda_fail(e, "stream ordering");
    }
    void destroy()
    {
        if (stream) cudaStreamSynchronize(stream);
        arena.stream = stream;
        arena.release();
        if (stream) cudaStreamSynchronize(stream);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (ev_legacy) cudaEventDestroy(ev_legacy);
        for (auto& ev : sev)
            if (ev) cudaEventDestroy(ev), ev = nullptr;
        for (auto& ev : cev)
            if (ev) cudaEventDestroy(ev), ev = nullptr;
        if (copy) cudaStreamSynchronize(copy), cudaStreamDestroy(copy), copy = nullptr;
        if (stream && own_stream) cudaStreamDestroy(stream);
        stream = nullptr;
        ev0 = ev1 = nullptr;
    }
};

thread_local std::unique_ptr<Workspace> t_ws;
thread_local float t_stage_ms[4] = {0, 0, 0, 0};   // delay model, F stage, X stage, output

Workspace* thread_ws(int* rc)
{
    if (!t_ws) t_ws.reset(new Workspace());
    *rc = t_ws->init();
    return *rc ? nullptr : t_ws.get();
}

long long budget_bytes()
{
    long long b = g_budget.load();
    if (b > 0) return b;
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) return 0;
    return (long long)(0.9 * (double)fr);
}

// Admission limit for one job: an explicit budget is a hard per-job cap;
// otherwise 90% of free device memory plus what this workspace already holds.
long long job_limit(const Workspace& ws)
{
    long long b = g_budget.load();
    if (b > 0) return b;
    return budget_bytes() + (long long)ws.arena.capacity();
}

// Staging helper: host buffers are copied through the workspace; device
// buffers are used in place.
struct Job {
    Workspace& ws;
    bool host;
    int err = 0;
    Job(Workspace& w, bool h) : ws(w), host(h)
    {
        ws.outs.clear();
        ws.arena.stream = ws.stream;        // scratch is ordered on the stream the job runs on
    }
    void* scratch(size_t bytes)
    {
        cudaError_t e = cudaSuccess;
        void* p = ws.arena.take(bytes, &e);
        if (!p && !err) err = cuda_fail(e, "workspace allocation");
        return p;
    }
    const void* in(const void* p, size_t bytes)
    {
        if (!host || !p || bytes == 0) return p;
        void* d = scratch(bytes);
        if (d && !err) {
            cudaError_t e = cudaMemcpyAsync(d, p, bytes, cudaMemcpyHostToDevice, ws.stream);
            if (e != cudaSuccess) err = cuda_fail(e, "host to device copy");
        }
        return d;
    }
    void* out(void* p, size_t bytes, bool load_existing)
    {
        if (!host || !p || bytes == 0) return p;
        void* d = scratch(bytes);
        if (d && !err) {
            if (load_existing) {
                cudaError_t e = cudaMemcpyAsync(d, p, bytes, cudaMemcpyHostToDevice, ws.stream);
                if (e != cudaSuccess) err = cuda_fail(e, "host to device copy");
            }
            ws.outs.push_back({p, d, bytes});
        }
        return d;
    }
    int finish(bool sync = true)
    {
        if (err) {
            cudaStreamSynchronize(ws.stream);
            ws.arena.reset();
            return err;
        }
        for (auto& o : ws.outs) {
            cudaError_t e = cudaMemcpyAsync(o.host, o.dev, o.bytes, cudaMemcpyDeviceToHost, ws.stream);
            if (e != cudaSuccess) return cuda_fail(e, "device to host copy");
        }
        ws.outs.clear();
        if (!sync) return 0;
        cudaError_t e = cudaStreamSynchronize(ws.stream);
        ws.arena.reset();
        if (e != cudaSuccess) return cuda_fail(e, "kernel execution");
        return 0;
    }
};

bool pick_levels(int format, const float* custom, float out[4])
{
    static const float mk5b[4] = {-3.3359f, 1.0f, -1.0f, 3.3359f};
    static const float twob[4] = {1.0f, -1.0f, 3.3359f, -3.3359f};
    static const float offb[4] = {-3.336f, -1.0f, 1.0f, 3.336f};
    static const float vdif[4] = {-3.3359f, -1.0f, 1.0f, 3.3359f};
    if (custom) {
        std::memcpy(out, custom, 4 * sizeof(float));
        return true;
    }
    switch (format & 0xff) {
        case CELLSPE_LEVELS_MARK5B: std::memcpy(out, mk5b, sizeof mk5b); return true;
        case CELLSPE_LEVELS_TWOBIT: std::memcpy(out, twob, sizeof twob); return true;
        case CELLSPE_LEVELS_OFFSET_BINARY: std::memcpy(out, offb, sizeof offb); return true;
        case CELLSPE_LEVELS_VDIF: std::memcpy(out, vdif, sizeof vdif); return true;
        default: return false;
    }
}

bool pow2(long long n) { return n > 0 && (n & (n - 1)) == 0; }

// ---------------------------------------------------------------------------
// engine operations (shared by the direct API and the task runtime)
// ---------------------------------------------------------------------------
int op_unpack(Workspace& ws, bool host, const void* raw, long long nsamp, int nchan, int format,
              const float* custom, float* out)
{
    float lut[4];
    if (!pick_levels(format, custom, lut)) return set_err(CELLSPE_ERR_ARG, "unpack: unknown level table");
    if (nsamp < 0 || !raw || !out) return set_err(CELLSPE_ERR_ARG, "unpack: bad arguments");
    bool msb = (format & CELLSPE_UNPACK_MSB_FIRST) != 0;
    size_t in_bytes = (size_t)((nsamp * nchan * 2 + 7) / 8);
    size_t out_bytes = (size_t)nsamp * nchan * sizeof(float);
    Job j(ws, host);
    const void* d_in = j.in(raw, in_bytes);
    float* d_out = (float*)j.out(out, out_bytes, false);
    if (!j.err) {
        int rc = map_rc(cs_unpack2bit(d_in, nsamp, nchan, msb, lut, d_out, ws.stream), "unpack");
        if (rc) j.err = rc;
    }
    return j.finish();
}

int op_fft(Workspace& ws, bool host, const void* in, void* out, int n, long long batch, bool real)
{
    if (!in || !out || batch < 0 || !pow2(n)) return set_err(CELLSPE_ERR_ARG, "fft: bad arguments");
    size_t in_bytes = real ? (size_t)n * batch * 4 : (size_t)n * batch * 8;
    size_t out_bytes = real ? (size_t)(n / 2 + 1) * batch * 8 : (size_t)n * batch * 8;
    Job j(ws, host);
    const void* d_in = j.in(in, in_bytes);
    void* d_out = j.out(out, out_bytes, false);
    if (!j.err) {
        int rc = real ? cs_rfft_batch((const float*)d_in, (float2*)d_out, n, batch, ws.stream)
                      : cs_cfft_batch((const float2*)d_in, (float2*)d_out, n, batch, ws.stream);
        rc = map_rc(rc, "fft");
        if (rc) j.err = rc;
    }
    return j.finish();
}

// Real FFT with IPP Perm-packed rows: the bins go to workspace scratch, then
// one packing pass writes [R0, R_{n/2}, Re 1, Im 1, ...] per row.
int op_fft_perm(Workspace& ws, bool host, const float* in, float* out, int n, long long batch)
{
    if (!in || !out || batch < 0 || !pow2(n) || n < 32 || n > 32768)
        return set_err(CELLSPE_ERR_ARG, "fft_r2c_perm: need n a power of two in [32, 32768]");
    Job j(ws, host);
    const void* d_in = j.in(in, (size_t)n * batch * 4);
    void* bins = j.scratch((size_t)(n / 2 + 1) * batch * 8);
    float* d_out = (float*)j.out(out, (size_t)n * batch * 4, false);
    if (!j.err) {
        int rc = map_rc(cs_rfft_batch((const float*)d_in, (float2*)bins, n, batch, ws.stream), "fft_r2c_perm");
        if (!rc) rc = map_rc(cs_perm_pack((const float2*)bins, d_out, n, batch, ws.stream), "fft_r2c_perm pack");
        if (rc) j.err = rc;
    }
    return j.finish();
}

int op_xmac(Workspace& ws, bool host, const void* spectra, int S, int C, int K, void* vis, int accumulate)
{
    if (!spectra || !vis || S <= 0 || C <= 0 || K <= 0) return set_err(CELLSPE_ERR_ARG, "xmac: bad arguments");
    long long P = (long long)S * (S + 1) / 2;
    Job j(ws, host);
    const void* d_sp = j.in(spectra, (size_t)C * S * K * 8);
    void* d_vis = j.out(vis, (size_t)C * P * 8, accumulate != 0);
    if (!j.err) {
        int rc = map_rc(cs_xmac_f32((const float2*)d_sp, S, C, K, K, (float2*)d_vis, accumulate, ws.stream), "xmac");
        if (rc) j.err = rc;
    }
    return j.finish();
}

int op_xmac_f16(Workspace& ws, bool host, const void* spectra, int S, int C, int K, void* vis, int accumulate)
{
    if (!spectra || !vis || S <= 0 || C <= 0 || K <= 0 || K % 8)
        return set_err(CELLSPE_ERR_ARG, "xmac_f16: bad arguments (K must be a multiple of 8)");
    long long P = (long long)S * (S + 1) / 2;
    Job j(ws, host);
    const void* d_sp = j.in(spectra, (size_t)C * 2 * S * K * 2);
    void* d_vis = j.out(vis, (size_t)C * P * 8, accumulate != 0);
    if (!j.err) {
        int rc = map_rc(cs_xmac_tc_f16(d_sp, S, C, K, K, (float2*)d_vis, nullptr, 0, accumulate, ws.stream), "xmac_f16");
        if (rc) j.err = rc;
    }
    int rc = j.finish();
    if (!rc) {
        unsigned code = 0;
        if (cs_xmac_tc_status(&code) != 0 || code != 0)
            rc = set_err(CELLSPE_ERR_CUDA, "xmac_f16: tensor-core pipeline wait timed out (code " + std::to_string(code) + ")");
    }
    return rc;
}

int op_xmac_i8(Workspace& ws, bool host, const void* planes, const float* scale, int S, int C, int K, void* vis,
               int accumulate)
{
    if (!planes || !scale || !vis || S <= 0 || C <= 0 || K <= 0 || K % 16 || K > 65536)
        return set_err(CELLSPE_ERR_ARG, "xmac_i8: bad arguments (K must be a multiple of 16, at most 65536)");
    long long P = (long long)S * (S + 1) / 2;
    Job j(ws, host);
    const void* d_pl = j.in(planes, (size_t)C * 2 * S * K);
    const void* d_sc = j.in(scale, (size_t)S * C * 4);
    void* d_vis = j.out(vis, (size_t)C * P * 8, accumulate != 0);
    if (!j.err) {
        int rc = map_rc(cs_xmac_i8((const int8_t*)d_pl, S, C, K, K, (float2*)d_vis, (const float*)d_sc, C, accumulate,
                                   ws.stream), "xmac_i8");
        if (rc) j.err = rc;
    }
    return j.finish();
}

// Row pitch (elements) of the internal spectra between the F and X stages:
// K + 64 for long rows.  Unpadded, the F stage's corner-turn writes land on
// rows a power-of-two number of bytes apart (4 MiB at 512 inputs x 4096
// segments), which measured 16% slower; the pad keeps rows 128-byte aligned
// for the X stage's TMA loads and costs at most 25% memory at K = 256 (1.6%
// at K = 4096).
long long spectra_pitch(long long K) { return K >= 256 ? K + 64 : K; }

long long fx_bytes(const cellspe_fx_params* p, bool with_poly)
{
    long long S = p->n_inputs, N = p->fft_points, K = p->n_segments, C = N / 2;
    long long P = S * (S + 1) / 2;
    bool host = p->memory == CELLSPE_MEM_HOST;
    long long b = 0;
    if (host) b += align256(S * p->bytes_per_input);
    if (with_poly) b += align256(S * 32) + 3 * align256(S * K * 4);
    const bool f32 = p->x_mode != CELLSPE_X_TC_FP16;   // FP32 spectra (FP32 and INT8 X stages)
    b += align256(C * S * spectra_pitch(K) * (f32 ? 8 : 4));
    if (N >= 4096) b += align256(C * S * K * (f32 ? 8 : 4));   // segment-major spectra
    if (p->x_mode == CELLSPE_X_INT8) b += align256(C * 2 * S * spectra_pitch(K)) + align256(S * C * 4);
    bool stage_vis = host || p->vis_order == CELLSPE_VIS_BASELINE_MAJOR || p->accumulate;
    if (stage_vis) b += 3 * align256(C * P * 8);
    if (p->x_mode == CELLSPE_X_TC_FP16) b += 2 * align256(S * C * 4);
    return b;
}

int op_fx(Workspace& ws, const cellspe_fx_params* p, const void* raw, const double* poly, void* vis, bool sync)
{
    if (!p || !raw || !vis) return set_err(CELLSPE_ERR_ARG, "fx: null argument");
    const int S = p->n_inputs, N = p->fft_points, K = p->n_segments, C = N / 2;
    if (S <= 0 || K <= 0 || !pow2(N) || N < 512 || N > 32768)
        return set_err(CELLSPE_ERR_ARG, "fx: need S > 0, K > 0, N a power of two in [512, 32768]");
    if (p->bytes_per_input <= 0 || p->bytes_per_input % 16)
        return set_err(CELLSPE_ERR_ARG, "fx: bytes_per_input must be a positive multiple of 16");
    if (!poly && (p->start_sample < 0 || p->start_sample + (long long)K * N > p->bytes_per_input * 4))
        return set_err(CELLSPE_ERR_ARG, "fx: segments run past the end of the input");
    if (p->x_mode != CELLSPE_X_FP32 && p->x_mode != CELLSPE_X_TC_FP16 && p->x_mode != CELLSPE_X_INT8)
        return set_err(CELLSPE_ERR_ARG, "fx: unknown x_mode");
    if (p->x_mode == CELLSPE_X_INT8 && (K % 16 || K > 65536))
        return set_err(CELLSPE_ERR_ARG, "fx: the INT8 X stage needs K a multiple of 16, at most 65536");
    if (poly && !(p->sample_rate_hz > 0)) return set_err(CELLSPE_ERR_ARG, "fx: delay model needs sample_rate_hz");
    float lut[4];
    if (!pick_levels(p->levels, p->custom_levels, lut)) return set_err(CELLSPE_ERR_ARG, "fx: unknown level table");
    long long need = fx_bytes(p, poly != nullptr);
    long long budget = job_limit(ws);
    if (need > budget)
        return set_err(CELLSPE_ERR_NOMEM, "fx: job needs " + std::to_string(need) + " device bytes, budget " +
                                              std::to_string(budget));
    const bool host = p->memory == CELLSPE_MEM_HOST;
    const long long P = (long long)S * (S + 1) / 2;
    const long long bpi = p->bytes_per_input;
    // Host buffers of large jobs move in chunks on the copy stream: input
    // blocks of inputs while the F stage transforms the blocks already there,
    // channel blocks of visibilities while the X stage computes later ones.
    // (Kernels reading and writing page-locked host buffers in place over the
    // CPU-GPU link measured slower here: the link carries ~193 GB/s to the host
    // and ~211 GB/s from it whether copy engines or SMs drive it, and SM
    // writes then stretch the X stage.)
    const int nsc = (host && sync && S * bpi >= (64LL << 20)) ? std::min(S, PIPE_IN) : 1;
    const bool stream_out = nsc > 1 && !p->accumulate && p->vis_order == CELLSPE_VIS_CHANNEL_MAJOR;
    const int ncb = stream_out ? std::min(C, PIPE_OUT) : 1;
    Job j(ws, host);
    const uint8_t* d_raw = nsc > 1 ? (const uint8_t*)j.scratch((size_t)(S * bpi))
                                   : (const uint8_t*)j.in(raw, (size_t)(S * bpi));
    if (nsc > 1 && !j.err) {
        // the copy stream starts after everything queued before this job
        cudaEventRecord(ws.cev[PIPE_IN + PIPE_OUT], ws.stream);
        cudaStreamWaitEvent(ws.copy, ws.cev[PIPE_IN + PIPE_OUT], 0);
        std::unique_lock<std::mutex> chain_lk;
        if (ws.chain) {
            chain_lk = std::unique_lock<std::mutex>(ws.chain->mu);
            if (ws.chain->valid) cudaStreamWaitEvent(ws.copy, ws.chain->in_done, 0);
        }
        for (int i = 0; i < nsc && !j.err; i++) {
            const long long s0 = (long long)S * i / nsc, s1 = (long long)S * (i + 1) / nsc;
            cudaError_t e = cudaMemcpyAsync((void*)(d_raw + s0 * bpi), (const uint8_t*)raw + s0 * bpi,
                                            (size_t)((s1 - s0) * bpi), cudaMemcpyHostToDevice, ws.copy);
            if (e == cudaSuccess) e = cudaEventRecord(ws.cev[i], ws.copy);
            if (e != cudaSuccess) j.err = cuda_fail(e, "host to device copy");
        }
        if (ws.chain && !j.err) {
            ws.chain->valid = cudaEventRecord(ws.chain->in_done, ws.copy) == cudaSuccess;
        }
    }
    if (sync) cudaEventRecord(ws.sev[0], ws.stream);
    CsFStageArgs fa{};
    fa.raw = d_raw;
    fa.bytes_per_input = p->bytes_per_input;
    fa.S = S; fa.N = N; fa.K = K;
    fa.start_sample = p->start_sample;
    std::memcpy(fa.lut, lut, sizeof lut);
    fa.msb_first = (p->levels & CELLSPE_UNPACK_MSB_FIRST) ? 1 : 0;
    fa.format = p->x_mode == CELLSPE_X_TC_FP16 ? CS_SPECTRA_F16 : CS_SPECTRA_F32;
    if (poly) {
        const double* d_poly = (const double*)j.in(poly, (size_t)S * 4 * sizeof(double));
        CsDelayState ds;
        ds.shift = (int32_t*)j.scratch((size_t)S * K * 4);
        ds.phase0 = (float*)j.scratch((size_t)S * K * 4);
        ds.dphase = (float*)j.scratch((size_t)S * K * 4);
        if (!j.err) {
            int rc = map_rc(cs_delay_state(d_poly, S, N, K, p->sample_rate_hz, p->lo_freq_hz, ds, ws.stream), "delay model");
            if (rc) j.err = rc;
        }
        fa.shift = ds.shift; fa.phase0 = ds.phase0; fa.dphase = ds.dphase;
    }
    const float* d_inv_scale = nullptr;
    if (p->x_mode == CELLSPE_X_TC_FP16 && p->channel_scale) {
        // F stage multiplies channel c of input s by scale[s][c] before the
        // FP16 cast; the X-stage epilogue divides V_ij by scale_i * scale_j.
        fa.scale = (const float*)j.in(p->channel_scale, (size_t)S * C * 4);
        float* inv = (float*)j.scratch((size_t)S * C * 4);
        if (!j.err) {
            int rc = map_rc(cs_reciprocal(fa.scale, inv, (int64_t)S * C, ws.stream), "scale");
            if (rc) j.err = rc;
        }
        d_inv_scale = inv;
    }
    const int kp = (int)spectra_pitch(K);
    fa.kp = kp;
    // FP16, N = 2048: 128-byte runs per 32 segments, k-blocked (1) or
    // channel-grouped k-blocked (2, the warp-specialised F stage)
    fa.kblock = cs_fstage_layout(fa);
    fa.out = j.scratch((size_t)C * S * kp * (fa.format == CS_SPECTRA_F32 ? 8 : 4));
    if (sync) cudaEventRecord(ws.sev[1], ws.stream);
    // bytes of one spectra element: F32 rows [C][S][kp] of float2, F16 rows [C][2][S][kp] of half
    const long long el_bytes = fa.format == CS_SPECTRA_F32 ? 8 : 2;
    // 4096-point and longer transforms stage at most 4 segments per CTA, so
    // their spectra are written segment-major and transposed in 64 x 64 tiles
    const bool segmaj = N >= 4096;
    const long long seg_bytes = fa.format == CS_SPECTRA_F32 ? 8 : 4;       // one channel of one segment
    char* seg_tmp = segmaj ? (char*)j.scratch((size_t)((long long)S * K * C * seg_bytes)) : nullptr;
    for (int i = 0; i < nsc && !j.err; i++) {
        CsFStageArgs fb = fa;
        long long s0 = 0, s1 = S;
        if (nsc > 1) {
            s0 = (long long)S * i / nsc, s1 = (long long)S * (i + 1) / nsc;
            cudaStreamWaitEvent(ws.stream, ws.cev[i], 0);
            fb.raw = d_raw + s0 * bpi;
            fb.S = (int)(s1 - s0);
            fb.S_out = S;
            // input s0's row in every (c, plane) block, its k-blocked rows in every
            // channel, or its runs in every channel group
            fb.out = (char*)fa.out + s0 * kp * el_bytes * (fa.kblock == 2 ? 32 : fa.kblock ? 2 : 1);
            if (fa.shift) fb.shift = fa.shift + s0 * K;
            if (fa.phase0) fb.phase0 = fa.phase0 + s0 * K, fb.dphase = fa.dphase + s0 * K;
            if (fa.scale) fb.scale = fa.scale + s0 * C;
        }
        void* rows_out = fb.out;
        if (segmaj) {
            fb.seg_major = 1;
            fb.out = seg_tmp + s0 * K * C * seg_bytes;
        }
        int rc = map_rc(cs_fx_fstage(fb, ws.stream), "F stage");
        if (!rc && segmaj)
            rc = map_rc(cs_spectra_transpose(fb.out, (int)(s1 - s0), K, C, kp, S, fa.format, rows_out, ws.stream),
                        "spectra transpose");
        if (rc) j.err = rc;
    }
    // INT8 X stage: FP32 spectra -> int8 planes [C][2][S][kp] and per-row scales
    int8_t* i8_planes = nullptr;
    float* i8_scale = nullptr;
    if (p->x_mode == CELLSPE_X_INT8 && !j.err) {
        i8_planes = (int8_t*)j.scratch((size_t)C * 2 * S * kp);
        i8_scale = (float*)j.scratch((size_t)S * C * 4);
        if (!j.err) {
            int rc = map_rc(cs_quantise_i8((const float2*)fa.out, S, C, K, kp, i8_planes, i8_scale, ws.stream), "INT8 quantise");
            if (rc) j.err = rc;
        }
    }
    if (sync) cudaEventRecord(ws.sev[2], ws.stream);
    // X stage into a channel-major buffer
    const bool direct = !host && p->vis_order == CELLSPE_VIS_CHANNEL_MAJOR && !p->accumulate;
    float2* vis_cp = direct ? (float2*)vis : (float2*)j.scratch((size_t)C * P * 8);
    for (int b = 0; b < ncb && !j.err; b++) {
        // streamed output: a small first block (1/16 of the channels) starts the
        // copy out early; the rest in equal blocks
        // (channel-grouped spectra: block bounds on whole groups of 16 channels)
        auto cbound = [&](int i) -> long long {
            if (ncb == 1) return i ? C : 0;
            if (i == ncb) return C;
            const long long first = std::max(1LL, (long long)C / 16);
            const long long c = i == 0 ? 0 : first + (long long)(C - first) * (i - 1) / (ncb - 1);
            return fa.kblock == 2 ? c / 16 * 16 : c;
        };
        const long long c0 = cbound(b), c1 = cbound(b + 1), cn = c1 - c0;
        if (cn <= 0) continue;
        int rc;
        if (p->x_mode == CELLSPE_X_FP32)
            rc = cs_xmac_f32((const float2*)fa.out + c0 * S * kp, S, (int)cn, K, kp, vis_cp + c0 * P, 0, ws.stream);
        else if (p->x_mode == CELLSPE_X_INT8)
            rc = cs_xmac_i8(i8_planes + c0 * 2 * S * kp, S, (int)cn, K, kp, vis_cp + c0 * P, i8_scale + c0, C, 0,
                            ws.stream);
        else
            rc = cs_xmac_tc_f16((const uint16_t*)fa.out + c0 * 2 * S * kp, S, (int)cn, K, kp, vis_cp + c0 * P,
                                d_inv_scale ? d_inv_scale + c0 : nullptr, C, 0, ws.stream, fa.kblock);
        rc = map_rc(rc, "X stage");
        if (!rc && stream_out) {
            cudaError_t e = cudaEventRecord(ws.cev[PIPE_IN + b], ws.stream);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(ws.copy, ws.cev[PIPE_IN + b], 0);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync((float2*)vis + c0 * P, vis_cp + c0 * P, (size_t)(cn * P * 8), cudaMemcpyDeviceToHost,
                                    ws.copy);
            if (e != cudaSuccess) rc = cuda_fail(e, "device to host copy");
        }
        if (rc) j.err = rc;
    }
    if (nsc > 1) {
        // the job ends when the copy stream's work has ended too
        cudaEventRecord(ws.cev[PIPE_IN + PIPE_OUT + 1], ws.copy);
        cudaStreamWaitEvent(ws.stream, ws.cev[PIPE_IN + PIPE_OUT + 1], 0);
    }
    if (sync) cudaEventRecord(ws.sev[3], ws.stream);
    if (!direct && !stream_out && !j.err) {
        float2* result = vis_cp;
        if (p->vis_order == CELLSPE_VIS_BASELINE_MAJOR) {
            float2* t = (float2*)j.scratch((size_t)C * P * 8);
            if (!j.err) {
                int rc = map_rc(cs_vis_to_baseline_major(vis_cp, t, C, P, ws.stream), "transpose");
                if (rc) j.err = rc;
            }
            result = t;
        }
        if (!j.err) {
            if (p->accumulate) {
                float2* old = (float2*)j.out(vis, (size_t)C * P * 8, true);
                if (!j.err) {
                    int rc = map_rc(cs_cadd(old, result, old, C * P, ws.stream), "accumulate");
                    if (rc) j.err = rc;
                }
            } else if (host) {
                ws.outs.push_back({vis, result, (size_t)C * P * 8});
            } else {
                cudaError_t e = cudaMemcpyAsync(vis, result, (size_t)C * P * 8, cudaMemcpyDeviceToDevice, ws.stream);
                if (e != cudaSuccess) j.err = cuda_fail(e, "result copy");
            }
        }
    }
    if (sync) cudaEventRecord(ws.sev[4], ws.stream);
    // after a failure the copy stream may still hold copies into the workspace
    if (nsc > 1 && j.err) cudaStreamSynchronize(ws.copy);
    int rc = j.finish(sync);
    if (sync && !rc && p->x_mode == CELLSPE_X_TC_FP16) {
        unsigned code = 0;
        unsigned code32 = 0;
        if (cs_fstage_tc_status(&code) != 0 || code != 0 || cs_fstage_tc32_status(&code32) != 0 || code32 != 0)
            rc = set_err(CELLSPE_ERR_CUDA, "F stage: tensor-core pipeline wait timed out (code " +
                                               std::to_string(code | code32) + ")");
        else if (cs_xmac_tc_status(&code) != 0 || code != 0)
            rc = set_err(CELLSPE_ERR_CUDA, "X stage: tensor-core pipeline wait timed out (code " +
                                               std::to_string(code) + ")");
    }
    if (sync && !rc) {
        for (int i = 0; i < 4; i++) {
            float ms = 0.f;
            t_stage_ms[i] = cudaEventElapsedTime(&ms, ws.sev[i], ws.sev[i + 1]) == cudaSuccess ? ms : -1.f;
        }
    }
    return rc;
}

constexpr long long M5B_FRAME = 10016, M5B_PAYLOAD = 10000;

// Sample-time groups of 16 per channel plane for a framed Mark5B buffer: every
// sample time of the frames that fit, rounded up to 64 so each plane is a
// multiple of 16 bytes.
long long m5b_groups(long long raw_bytes, int nch)
{
    const long long spf = M5B_PAYLOAD / (nch / 4);
    const long long nsamp = (raw_bytes / M5B_FRAME) * spf;
    return ((nsamp + 63) / 64) * 4;
}

// ---- framed Mark5B / VDIF ---------------------------------------------------
// Header fields as FileSource::locateFirstHeader (FileSource.cpp:330-333) and
// the mark5access frame-number field (bits 0..14 of header word 1).
void m5b_header_info(const uint8_t h[16], cellspe_mark5b_info* info)
{
    info->mjd = 56000 + (h[11] >> 4) * 100 + (h[11] & 15) * 10 + (h[10] >> 4);
    info->seconds = (h[10] & 15) * 10000 + (h[9] >> 4) * 1000 + (h[9] & 15) * 100 + (h[8] >> 4) * 10 + (h[8] & 15);
    info->frame_number = h[4] | ((h[5] & 0x7f) << 8);
}

// A framed stream staged on the device with its frame geometry and the valid
// byte range of every complete frame (Mark5B: the first-frame offset stays on
// the device in d_off; VDIF: frames from byte 0, d_off null).
struct Located {
    const uint8_t* d_framed = nullptr;
    int* d_off = nullptr;
    int2* d_ranges = nullptr;
    unsigned long long* d_blanked = nullptr;
    CsFraming fmt{};
    long long off = -1, frames = 0, bytes = 0;
};

CsFraming m5b_framing(int nch) { return CsFraming{M5B_FRAME, (int)M5B_PAYLOAD, 16, 16, nch}; }

// Reads n bytes at offset off of a host or device buffer into h.
int read_head(Workspace& ws, bool host, const void* src, const uint8_t* d_src, long long off, void* h, size_t n,
              const char* what)
{
    if (host) {
        std::memcpy(h, (const uint8_t*)src + off, n);
        return 0;
    }
    cudaError_t e = cudaMemcpyAsync(h, d_src + off, n, cudaMemcpyDeviceToHost, ws.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ws.stream);
    return e == cudaSuccess ? 0 : cuda_fail(e, what);
}

// Stages the framed bytes, finds the first frame and the valid ranges of
// every frame, and brings the frame offset back (the callers need the frame
// count on the host).  Fills info except good_samples.
int m5b_locate(Workspace& ws, Job& j, const void* framed, long long bytes, int nch, Located& L,
               cellspe_mark5b_info* info)
{
    const long long nmax = bytes / M5B_FRAME;
    L.fmt = m5b_framing(nch);
    L.bytes = bytes;
    L.d_framed = (const uint8_t*)j.in(framed, (size_t)bytes);
    L.d_off = (int*)j.scratch(sizeof(int));
    L.d_ranges = (int2*)j.scratch((size_t)nmax * sizeof(int2));
    if (j.err) return j.err;
    int rc = map_rc(cs_m5b_locate(L.d_framed, bytes, L.d_off, L.d_ranges, nmax, ws.stream), "frame search");
    if (rc) return rc;
    int off = 0;
    if ((rc = read_head(ws, false, nullptr, (const uint8_t*)L.d_off, 0, &off, sizeof off, "frame search"))) return rc;
    if (off < 0 || off >= (1 << 20)) return set_err(CELLSPE_ERR_ARG, "mark5b: no frame found in the first MiB");
    L.off = off;
    L.frames = (bytes - off) / M5B_FRAME;
    if (info) {
        uint8_t h[16];
        if ((rc = read_head(ws, j.host, framed, L.d_framed, off, h, 16, "header read"))) return rc;
        info->first_frame_offset = off;
        info->frames = L.frames;
        info->good_samples = 0;
        m5b_header_info(h, info);
        info->reserved = 0;
    }
    return 0;
}

// MJD of the VDIF reference epoch e: 1 January (even e) or 1 July (odd e) of
// year 2000 + e / 2, counted from the proleptic Gregorian calendar (days
// since 1 March of year 0 shifted to MJD 0 = 1858-11-17).
int vdif_epoch_mjd(int e)
{
    long y = 2000 + e / 2;
    const int month = (e & 1) ? 7 : 1;
    if (month <= 2) y -= 1;
    const long mp = month > 2 ? month - 3 : month + 9;           // months since March
    const long days = 365 * y + y / 4 - y / 100 + y / 400 + (153 * mp + 2) / 5;  // day 1 of the month
    return (int)(days - 678881);                                 // 1858-11-17 = day 678881
}

// The stream geometry and the header-time model of a VDIF buffer opened as
// mark5access does with the format "VDIF_<payload>-<mbps>-<nch>-2"
// (mark5_format_vdif_init, format_vdif.c:2121-2257): frame length and legacy
// flag from the first header; frame duration payload * 8000 / mbps ns with
// the smallest power-of-two granularity (< 128) that makes a whole number of
// ns (32-bit products, as the library computes them); frame 0's payload 32
// bytes into the frame whatever the header length.
int vdif_model(const uint8_t h[32], long long bytes, int nch, int mbps, CsVdifClock& c, cellspe_vdif_info* info,
               const char* who)
{
    const std::string w(who);
    if (!(nch == 1 || nch == 2 || nch == 4 || nch == 8 || nch == 16))
        return set_err(CELLSPE_ERR_ARG, w + ": nchan must be 1, 2, 4, 8 or 16 (2-bit VDIF)");
    if (mbps <= 0) return set_err(CELLSPE_ERR_ARG, w + ": Mbps must be positive");
    auto word = [&](int k) {
        return (uint32_t)h[4 * k] | ((uint32_t)h[4 * k + 1] << 8) | ((uint32_t)h[4 * k + 2] << 16) |
               ((uint32_t)h[4 * k + 3] << 24);
    };
    const int hsize = (h[3] & 0x40) ? 16 : 32;
    const long long frame = (long long)(word(2) & 0x00FFFFFF) * 8;
    const long long payload = frame - hsize;
    if (payload < 8) return set_err(CELLSPE_ERR_ARG, w + ": first VDIF header gives no payload");
    if (payload * 8000 > INT32_MAX) return set_err(CELLSPE_ERR_UNSUPPORTED, w + ": VDIF payload above 268435 bytes");
    if (payload * 4 % nch) return set_err(CELLSPE_ERR_ARG, w + ": payload does not hold whole sample times");
    if (bytes < 2 * frame) return set_err(CELLSPE_ERR_ARG, w + ": fewer than two VDIF frames of input");
    c = CsVdifClock{};
    c.fmt = CsFraming{frame, (int)payload, hsize, 32, nch};
    const int num = (int)(payload * 8000), den = mbps;
    c.frame_ns = (double)num / (double)den;
    int g = 1;
    for (; g < 128; g *= 2)
        if ((int32_t)((uint32_t)g * (uint32_t)num) % den == 0) break;
    if (g >= 128) g = 1;
    c.granularity = g;
    const int gframe_ns = (int)(g * c.frame_ns + 0.5);
    c.step_ns = gframe_ns / g;
    for (int e = 0; e < 64; e++) c.epoch_mjd[e] = vdif_epoch_mjd(e);
    const uint32_t w0 = word(0), w1 = word(1);
    int sec = (int)(w0 & 0x3FFFFFFF);
    const int days = sec / 86400;
    sec -= days * 86400;
    c.mjd0 = days + c.epoch_mjd[(w1 >> 24) & 0x3F];
    c.sec0 = sec;
    c.ns0 = (int)((double)(w1 & 0x00FFFFFF) * c.frame_ns + 0.5);
    if (info) {
        *info = cellspe_vdif_info{};
        info->frames = bytes / frame;
        info->frame_bytes = (int)frame;
        info->header_bytes = hsize;
        info->mjd = c.mjd0;
        info->seconds = c.sec0;
        info->ns = c.ns0;
        info->frame_number = (int)(w1 & 0x00FFFFFF);
        info->nchan_header = 1 << ((word(2) >> 24) & 0x1F);
        info->thread_id = (int)((word(3) >> 16) & 0x3FF);
        info->station_id = (int)(word(3) & 0xFFFF);
    }
    return 0;
}

// Stages a VDIF buffer, builds its model from the first header and marks
// every frame used or blanked on the device.  Fills info except
// good_samples and blanked_frames (read back with the results).
int vdif_locate(Workspace& ws, Job& j, const void* framed, long long bytes, int nch, int mbps, Located& L,
                cellspe_vdif_info* info, const char* who)
{
    if (bytes < 32) return set_err(CELLSPE_ERR_ARG, std::string(who) + ": input shorter than a VDIF header");
    L.d_framed = (const uint8_t*)j.in(framed, (size_t)bytes);
    if (j.err) return j.err;
    uint8_t h[32];
    int rc = read_head(ws, j.host, framed, L.d_framed, 0, h, 32, "header read");
    if (rc) return rc;
    CsVdifClock c;
    if ((rc = vdif_model(h, bytes, nch, mbps, c, info, who))) return rc;
    L.fmt = c.fmt;
    L.off = 0;
    L.bytes = bytes;
    L.frames = bytes / c.fmt.frame_bytes;
    L.d_ranges = (int2*)j.scratch((size_t)L.frames * sizeof(int2));
    L.d_blanked = (unsigned long long*)j.scratch(sizeof(unsigned long long));
    if (j.err) return j.err;
    return map_rc(cs_vdif_locate(L.d_framed, bytes, c, L.d_ranges, L.frames, L.d_blanked, ws.stream), "VDIF frames");
}

int m5b_check(const void* framed, long long bytes, int nchan, const char* who)
{
    if (!framed) return set_err(CELLSPE_ERR_ARG, std::string(who) + ": null input");
    if (!(nchan == 4 || nchan == 8 || nchan == 16))
        return set_err(CELLSPE_ERR_ARG, std::string(who) + ": nchan must be 4, 8 or 16 (2-bit Mark5B)");
    if (bytes < 2 * M5B_FRAME) return set_err(CELLSPE_ERR_ARG, std::string(who) + ": fewer than two frames of input");
    return 0;
}

long long samples_per_frame(const CsFraming& f) { return (long long)f.payload_bytes * 4 / f.nch; }

// mark5_stream_decode over a located stream: the unblanked sample count, or
// -1 when the frames run out (nothing is written past the last frame, so the
// caller's values stay there).
int framed_decode(Workspace& ws, Job& j, const Located& L, long long nsamp, const float lut[4], float* out,
                  long long* good_out, const char* who)
{
    const bool runs_out = nsamp >= L.frames * samples_per_frame(L.fmt);
    float* d_out = (float*)j.out(out, (size_t)(nsamp * L.fmt.nch * 4), runs_out);
    auto* d_good = (unsigned long long*)j.scratch(sizeof(unsigned long long));
    unsigned long long good = 0, blanked = 0;
    if (!j.err) {
        int rc = map_rc(cs_framed_decode(L.d_framed, L.bytes, L.fmt, L.d_off, L.d_ranges, nsamp, lut, d_out, d_good, ws.stream), who);
        if (!rc) {
            cudaError_t e = cudaMemcpyAsync(&good, d_good, sizeof good, cudaMemcpyDeviceToHost, ws.stream);
            if (e == cudaSuccess && L.d_blanked)
                e = cudaMemcpyAsync(&blanked, L.d_blanked, sizeof blanked, cudaMemcpyDeviceToHost, ws.stream);
            if (e != cudaSuccess) rc = cuda_fail(e, who);
        }
        if (rc) j.err = rc;
    }
    int rc = j.finish();
    if (!rc) {
        good_out[0] = runs_out ? -1 : (long long)good;
        good_out[1] = (long long)blanked;
    }
    return rc;
}

int op_mark5b_decode(Workspace& ws, bool host, const void* framed, long long bytes, int nchan, long long nsamp,
                     float* out, cellspe_mark5b_info* info)
{
    if (int rc = m5b_check(framed, bytes, nchan, "mark5b_decode")) return rc;
    if (!out || nsamp <= 0) return set_err(CELLSPE_ERR_ARG, "mark5b_decode: bad output");
    const long long need = (host ? align256(bytes) + align256(nsamp * nchan * 4) : 0) + align256(bytes / M5B_FRAME * 8) + 512;
    if (need > job_limit(ws)) return set_err(CELLSPE_ERR_NOMEM, "mark5b_decode: job exceeds the device memory budget");
    cellspe_mark5b_info tmp{};
    if (!info) info = &tmp;
    Job j(ws, host);
    Located L;
    int rc = m5b_locate(ws, j, framed, bytes, nchan, L, info);
    if (rc) { j.err = rc; return j.finish(); }
    float lut[4];
    pick_levels(CELLSPE_LEVELS_MARK5B, nullptr, lut);
    long long res[2] = {0, 0};
    rc = framed_decode(ws, j, L, nsamp, lut, out, res, "mark5b decode");
    if (!rc) info->good_samples = res[0];
    return rc;
}

int op_vdif_decode(Workspace& ws, bool host, const void* framed, long long bytes, int nchan, int mbps,
                   long long nsamp, float* out, cellspe_vdif_info* info)
{
    if (!framed || !out || nsamp <= 0) return set_err(CELLSPE_ERR_ARG, "vdif_decode: null input or bad output");
    if (nchan < 4 && nchan > 0 && nsamp % (4 / nchan))
        return set_err(CELLSPE_ERR_ARG, "vdif_decode: nsamp must be a multiple of the samples per byte");
    const long long need = (host ? align256(bytes) + align256(nsamp * nchan * 4) : 0) + align256(bytes / 24 * 8) + 768;
    if (need > job_limit(ws)) return set_err(CELLSPE_ERR_NOMEM, "vdif_decode: job exceeds the device memory budget");
    cellspe_vdif_info tmp{};
    if (!info) info = &tmp;
    Job j(ws, host);
    Located L;
    int rc = vdif_locate(ws, j, framed, bytes, nchan, mbps, L, info, "vdif_decode");
    if (rc) { j.err = rc; return j.finish(); }
    float lut[4];
    pick_levels(CELLSPE_LEVELS_VDIF, nullptr, lut);
    long long res[2] = {0, 0};
    rc = framed_decode(ws, j, L, nsamp, lut, out, res, "vdif decode");
    if (!rc) {
        info->good_samples = res[0];
        info->blanked_frames = res[1];
    }
    return rc;
}

// Payloads (and validity mask) of `frames` located frames; frames = 0 takes
// them all.  Returns the blanked-frame count through *blanked when asked.
int framed_deframe(Workspace& ws, Job& j, const Located& L, long long frames, void* payload,
                   unsigned* mask, long long* blanked, const char* who)
{
    if (frames > L.frames) {
        j.err = set_err(CELLSPE_ERR_ARG, std::string(who) + ": fewer complete frames in the buffer than requested");
        return j.finish();
    }
    unsigned long long nb = 0;
    if (payload) {
        const long long spf = samples_per_frame(L.fmt);
        void* d_pay = j.out(payload, (size_t)(frames * L.fmt.payload_bytes), false);
        void* d_mask = mask ? j.out(mask, (size_t)((frames * spf + 31) / 32 * 4), false) : nullptr;
        if (!j.err) {
            int rc = map_rc(cs_framed_deframe(L.d_framed, L.bytes, L.fmt, L.d_off, L.d_ranges, frames, (uint8_t*)d_pay,
                                              (uint32_t*)d_mask, ws.stream), "deframe");
            if (rc) j.err = rc;
        }
    }
    if (!j.err && blanked && L.d_blanked) {
        cudaError_t e = cudaMemcpyAsync(&nb, L.d_blanked, sizeof nb, cudaMemcpyDeviceToHost, ws.stream);
        if (e != cudaSuccess) j.err = cuda_fail(e, who);
    }
    int rc = j.finish();
    if (!rc && blanked) *blanked = (long long)nb;
    return rc;
}

int op_mark5b_deframe(Workspace& ws, bool host, const void* framed, long long bytes, int nchan, long long frames,
                      void* payload, unsigned* mask, cellspe_mark5b_info* info)
{
    if (int rc = m5b_check(framed, bytes, nchan, "mark5b_deframe")) return rc;
    if (frames < 0) return set_err(CELLSPE_ERR_ARG, "mark5b_deframe: negative frame count");
    const long long nmax = bytes / M5B_FRAME, spf = M5B_PAYLOAD / (nchan / 4);
    const long long mwords_max = (nmax * spf + 31) / 32;
    const long long need = (host ? align256(bytes) + align256(nmax * M5B_PAYLOAD) + align256(mwords_max * 4) : 0) +
                           align256(nmax * 8) + 256;
    if (need > job_limit(ws)) return set_err(CELLSPE_ERR_NOMEM, "mark5b_deframe: job exceeds the device memory budget");
    cellspe_mark5b_info tmp{};
    if (!info) info = &tmp;
    Job j(ws, host);
    Located L;
    int rc = m5b_locate(ws, j, framed, bytes, nchan, L, info);
    if (rc) { j.err = rc; return j.finish(); }
    return framed_deframe(ws, j, L, frames == 0 ? L.frames : frames, payload, mask, nullptr, "mark5b_deframe");
}

int op_vdif_deframe(Workspace& ws, bool host, const void* framed, long long bytes, int nchan, int mbps,
                    long long frames, void* payload, unsigned* mask, cellspe_vdif_info* info)
{
    if (!framed) return set_err(CELLSPE_ERR_ARG, "vdif_deframe: null input");
    if (frames < 0) return set_err(CELLSPE_ERR_ARG, "vdif_deframe: negative frame count");
    const long long need = (host ? 2 * align256(bytes) + align256(bytes / 4 + 4) : 0) + align256(bytes / 24 * 8) + 512;
    if (need > job_limit(ws)) return set_err(CELLSPE_ERR_NOMEM, "vdif_deframe: job exceeds the device memory budget");
    cellspe_vdif_info tmp{};
    if (!info) info = &tmp;
    Job j(ws, host);
    Located L;
    int rc = vdif_locate(ws, j, framed, bytes, nchan, mbps, L, info, "vdif_deframe");
    if (rc) { j.err = rc; return j.finish(); }
    long long blanked = 0;
    rc = framed_deframe(ws, j, L, frames == 0 ? L.frames : frames, payload, mask, &blanked, "vdif_deframe");
    if (!rc) info->blanked_frames = blanked;
    return rc;
}

// Smallest VDIF frame the spectrometer takes (bounds its frame table).
constexpr long long VDIF_SPEC_MIN_FRAME = 528;

// Mbps of a VDIF stream carrying the spectrometer's subbands: 2 bits per
// sample, nsub channels at sample_rate_hz (0 when that is not a whole number).
int vdif_spec_mbps(const cellspe_spec_params* p)
{
    const double mbps = p->sample_rate_hz * 2.0 * p->n_subbands / 1e6;
    const long long r = std::llround(mbps);
    return (r > 0 && r < INT32_MAX && std::fabs(mbps - (double)r) < 1e-6) ? (int)r : 0;
}

long long spec_bytes(const cellspe_spec_params* p)
{
    CsSpecArgs a{};
    a.nsub = p->n_subbands; a.N = p->fft_points; a.overlap = p->overlap;
    a.ffts_per_spectrum = p->ffts_per_spectrum; a.nspec = p->n_spectra; a.tonebins = p->pcal_tonebins;
    long long b = align256(cs_spectrometer_scratch_floats(a) * 4);
    bool host = p->memory == CELLSPE_MEM_HOST;
    if (host) b += align256(p->raw_bytes);
    if (p->input_layout == CELLSPE_SPEC_INTERLEAVED && p->n_subbands > 1) b += align256(p->raw_bytes);
    if (p->input_layout == CELLSPE_SPEC_MARK5B_FRAMED) {
        const long long g = m5b_groups(p->raw_bytes, std::max(p->n_subbands, 4));
        b += align256(g * 4 * p->n_subbands) + align256((g + 1) / 2 * 4) + align256(p->raw_bytes / M5B_FRAME * 8) + 256;
    } else if (p->input_layout == CELLSPE_SPEC_VDIF_FRAMED) {
        // bounds: every byte a payload byte, frames of at least VDIF_SPEC_MIN_FRAME bytes
        const long long g = ((p->raw_bytes * 4 / p->n_subbands + 63) / 64) * 4;
        b += align256(g * 4 * p->n_subbands) + align256((g + 1) / 2 * 4) +
             align256(p->raw_bytes / VDIF_SPEC_MIN_FRAME * 8) + 512;
    }
    long long rows = (long long)p->n_subbands * p->n_spectra;
    if (host) b += align256(rows * (p->fft_points / 2 + 1) * 4) + 2 * align256(rows * std::max(p->pcal_tonebins, p->pcal_ntones) * 8);
    return b;
}

// Checks shared by the spectrometer entry points ("who" names the caller).
int spec_check(const cellspe_spec_params* p, const char* who)
{
    const std::string w(who);
    const int nsub = p->n_subbands;
    if (!(nsub == 1 || nsub == 4 || nsub == 8 || nsub == 16)) return set_err(CELLSPE_ERR_ARG, w + ": n_subbands must be 1, 4, 8 or 16");
    if (!pow2(p->fft_points) || p->fft_points < 1024 || p->fft_points > 65536)
        return set_err(CELLSPE_ERR_ARG, w + ": fft_points must be a power of two in [1024, 65536]");
    if (p->overlap < 1 || p->ffts_per_spectrum < 1 || p->n_spectra < 1 || p->fft_points % (16 * p->overlap))
        return set_err(CELLSPE_ERR_ARG, w + ": bad overlap, ffts_per_spectrum or n_spectra");
    if (p->window < 0 || p->window > 5)
        return set_err(CELLSPE_ERR_ARG, w + ": window must be 0 (none) .. 5 (Blackman)");
    // the phase-cal rotator is exp(-2 pi i offset n / fs): no rotator without a sample rate
    if (p->pcal_tonebins > 0 && !(p->sample_rate_hz > 0))
        return set_err(CELLSPE_ERR_ARG, w + ": phase-cal needs sample_rate_hz > 0");
    if (p->input_layout == CELLSPE_SPEC_MARK5B_FRAMED) {
        if (nsub == 1) return set_err(CELLSPE_ERR_ARG, w + ": framed Mark5B input needs 4, 8 or 16 subbands");
        if (p->raw_bytes < 2 * M5B_FRAME) return set_err(CELLSPE_ERR_ARG, w + ": framed input shorter than two frames");
        const long long avail = (p->raw_bytes / M5B_FRAME) * (M5B_PAYLOAD / (nsub / 4));
        if ((long long)p->n_spectra * p->ffts_per_spectrum * p->fft_points > avail)
            return set_err(CELLSPE_ERR_ARG, w + ": spectra need more samples than the frames hold");
    } else if (p->input_layout == CELLSPE_SPEC_VDIF_FRAMED) {
        if (!vdif_spec_mbps(p))
            return set_err(CELLSPE_ERR_ARG, w + ": VDIF input needs sample_rate_hz giving a whole number of Mbps");
        if (p->raw_bytes < 2 * VDIF_SPEC_MIN_FRAME) return set_err(CELLSPE_ERR_ARG, w + ": framed input shorter than two frames");
    } else if (p->input_layout != CELLSPE_SPEC_INTERLEAVED && p->input_layout != CELLSPE_SPEC_PLANES) {
        return set_err(CELLSPE_ERR_ARG, w + ": unknown input_layout");
    } else if (p->raw_bytes <= 0 || p->raw_bytes % (16 * nsub)) {
        return set_err(CELLSPE_ERR_ARG, w + ": raw_bytes must be a multiple of 16*n_subbands");
    }
    return 0;
}

// One recording on the device as per-subband 2-bit planes (+ validity mask
// for framed Mark5B): interleaved input is corner-turned, framed input is
// searched, deframed and corner-turned in one pass, planes are used in place.
struct SpecPlanes {
    const uint8_t* planes = nullptr;
    long long bytes_per_sub = 0;
    const uint32_t* vmask = nullptr;
};

SpecPlanes spec_planes(Workspace& ws, Job& j, const cellspe_spec_params* p, const void* raw)
{
    const int nsub = p->n_subbands;
    SpecPlanes r;
    const uint8_t* d_raw = (const uint8_t*)j.in(raw, (size_t)p->raw_bytes);
    r.planes = d_raw;
    r.bytes_per_sub = p->raw_bytes / nsub;
    if (p->input_layout == CELLSPE_SPEC_MARK5B_FRAMED) {
        const long long nframes = p->raw_bytes / M5B_FRAME, groups = m5b_groups(p->raw_bytes, nsub);
        void* pl = j.scratch((size_t)(groups * 4 * nsub));
        void* mk = j.scratch((size_t)((groups + 1) / 2 * 4));
        void* rg = j.scratch((size_t)(nframes * 8));
        void* off = j.scratch(sizeof(int));
        if (!j.err) {
            int rc = map_rc(cs_m5b_locate(d_raw, p->raw_bytes, (int*)off, (int2*)rg, nframes, ws.stream), "frame search");
            if (!rc)
                rc = map_rc(cs_framed_planes(d_raw, p->raw_bytes, m5b_framing(nsub), (const int*)off, (const int2*)rg,
                                             nframes, groups, (uint32_t*)pl, (uint32_t*)mk, ws.stream), "deframe");
            if (rc) j.err = rc;
        }
        r.planes = (const uint8_t*)pl;
        r.vmask = (const uint32_t*)mk;
        r.bytes_per_sub = groups * 4;
    } else if (p->input_layout == CELLSPE_SPEC_VDIF_FRAMED) {
        // the frame length comes from the first header: read it before sizing
        uint8_t h[32];
        CsVdifClock c;
        int rc = j.err;
        if (!rc) rc = read_head(ws, j.host, raw, d_raw, 0, h, 32, "header read");
        if (!rc) rc = vdif_model(h, p->raw_bytes, nsub, vdif_spec_mbps(p), c, nullptr, "spectrometer");
        if (!rc && c.fmt.frame_bytes < VDIF_SPEC_MIN_FRAME)
            rc = set_err(CELLSPE_ERR_ARG, "spectrometer: VDIF frames shorter than 528 bytes");
        const long long nframes = rc ? 0 : p->raw_bytes / c.fmt.frame_bytes;
        const long long spf = rc ? 0 : samples_per_frame(c.fmt);
        if (!rc && (long long)p->n_spectra * p->ffts_per_spectrum * p->fft_points > nframes * spf)
            rc = set_err(CELLSPE_ERR_ARG, "spectrometer: spectra need more samples than the frames hold");
        if (rc) {
            if (!j.err) j.err = rc;
            return r;
        }
        const long long groups = ((nframes * spf + 63) / 64) * 4;
        void* pl = j.scratch((size_t)(groups * 4 * nsub));
        void* mk = j.scratch((size_t)((groups + 1) / 2 * 4));
        void* rg = j.scratch((size_t)(nframes * 8));
        void* nb = j.scratch(sizeof(unsigned long long));
        if (!j.err) {
            rc = map_rc(cs_vdif_locate(d_raw, p->raw_bytes, c, (int2*)rg, nframes, (unsigned long long*)nb, ws.stream),
                        "VDIF frames");
            if (!rc)
                rc = map_rc(cs_framed_planes(d_raw, p->raw_bytes, c.fmt, nullptr, (const int2*)rg, nframes, groups,
                                             (uint32_t*)pl, (uint32_t*)mk, ws.stream), "deframe");
            if (rc) j.err = rc;
        }
        r.planes = (const uint8_t*)pl;
        r.vmask = (const uint32_t*)mk;
        r.bytes_per_sub = groups * 4;
    } else if (p->input_layout == CELLSPE_SPEC_INTERLEAVED && nsub > 1) {
        void* pl = j.scratch((size_t)p->raw_bytes);
        if (!j.err) {
            long long nsamp = p->raw_bytes * 4 / nsub;
            int rc = map_rc(cs_cornerturn2bit(d_raw, nsamp, nsub, pl, ws.stream), "corner turn");
            if (rc) j.err = rc;
        }
        r.planes = (const uint8_t*)pl;
    }
    return r;
}

CsSpecArgs spec_args(const cellspe_spec_params* p, const SpecPlanes& sp, const float lut[4])
{
    CsSpecArgs a{};
    a.planes = sp.planes; a.bytes_per_sub = sp.bytes_per_sub; a.nsub = p->n_subbands; a.N = p->fft_points;
    a.valid_mask = sp.vmask;
    a.overlap = p->overlap; a.window = p->window; a.ffts_per_spectrum = p->ffts_per_spectrum; a.nspec = p->n_spectra;
    std::memcpy(a.lut, lut, 4 * sizeof(float));
    a.tonebins = p->pcal_tonebins; a.rotatorlen = p->pcal_rotatorlen; a.ntones = p->pcal_ntones;
    a.pcal_offset_hz = p->pcal_offset_hz; a.fs_hz = p->sample_rate_hz;
    return a;
}

int op_spectrometer(Workspace& ws, const cellspe_spec_params* p, const void* raw, float* power, void* pcal_bins,
                    void* pcal_tones)
{
    if (!p || !raw || !power) return set_err(CELLSPE_ERR_ARG, "spectrometer: null argument");
    if (int rc = spec_check(p, "spectrometer")) return rc;
    if (p->pcal_tonebins > 0 && !pcal_bins) return set_err(CELLSPE_ERR_ARG, "spectrometer: pcal enabled without pcal_bins");
    float lut[4];
    if (!pick_levels(p->levels, p->custom_levels, lut)) return set_err(CELLSPE_ERR_ARG, "spectrometer: unknown level table");
    long long need = spec_bytes(p);
    long long budget = job_limit(ws);
    if (need > budget) return set_err(CELLSPE_ERR_NOMEM, "spectrometer: job exceeds the device memory budget");
    const bool host = p->memory == CELLSPE_MEM_HOST;
    Job j(ws, host);
    const SpecPlanes sp = spec_planes(ws, j, p, raw);
    CsSpecArgs a = spec_args(p, sp, lut);
    const long long rows = (long long)p->n_subbands * p->n_spectra;
    a.power = (float*)j.out(power, (size_t)rows * (p->fft_points / 2 + 1) * 4, false);
    if (a.tonebins > 0) {
        a.pcal_bins = (float2*)j.out(pcal_bins, (size_t)rows * a.tonebins * 8, false);
        a.pcal_tones = pcal_tones ? (float2*)j.out(pcal_tones, (size_t)rows * a.ntones * 8, false) : nullptr;
    }
    a.partial = (float*)j.scratch((size_t)cs_spectrometer_scratch_floats(a) * 4);
    if (!j.err) {
        int rc = map_rc(cs_spectrometer(a, ws.stream), "spectrometer");
        if (rc) j.err = rc;
    }
    return j.finish();
}

// Device bytes of one cross-polarisation job: both recordings' planes, the
// windows of one source and the spectra of both.
long long spec_xpol_bytes(const cellspe_spec_params* p)
{
    const long long N = p->fft_points, nb = N / 2 + 1;
    const long long nwin = (long long)p->n_spectra * (p->overlap * p->ffts_per_spectrum - (p->overlap - 1));
    cellspe_spec_params one = *p;
    one.n_subbands = p->n_subbands;
    long long b = 2 * spec_bytes(&one);
    b += align256(nwin * N * 4) + 2 * align256(nwin * nb * 8);
    b += align256(3LL * p->n_spectra * nb * 8);
    return b;
}

int op_spectrometer_xpol(Workspace& ws, const cellspe_spec_params* p, const void* raw0, const void* raw1, int ch0,
                         int ch1, float* power, void* xpol, void* pcal_bins)
{
    const char* who = "spectrometer_xpol";
    if (!p || !raw0 || !raw1 || !power || !xpol) return set_err(CELLSPE_ERR_ARG, "spectrometer_xpol: null argument");
    if (int rc = spec_check(p, who)) return rc;
    if (p->fft_points > 32768)
        return set_err(CELLSPE_ERR_UNSUPPORTED, "spectrometer_xpol: fft_points above 32768 are not supported");
    if (ch0 < 0 || ch0 >= p->n_subbands || ch1 < 0 || ch1 >= p->n_subbands)
        return set_err(CELLSPE_ERR_ARG, "spectrometer_xpol: channel outside the recording's subbands");
    if (p->pcal_tonebins > 0 && !pcal_bins) return set_err(CELLSPE_ERR_ARG, "spectrometer_xpol: pcal enabled without pcal_bins");
    float lut[4];
    if (!pick_levels(p->levels, p->custom_levels, lut)) return set_err(CELLSPE_ERR_ARG, "spectrometer_xpol: unknown level table");
    if (spec_xpol_bytes(p) > job_limit(ws))
        return set_err(CELLSPE_ERR_NOMEM, "spectrometer_xpol: job exceeds the device memory budget");
    const bool host = p->memory == CELLSPE_MEM_HOST;
    const int N = p->fft_points, nb = N / 2 + 1, nspec = p->n_spectra;
    const long long nwin = (long long)nspec * (p->overlap * p->ffts_per_spectrum - (p->overlap - 1));
    Job j(ws, host);
    SpecPlanes sp[2] = {spec_planes(ws, j, p, raw0), spec_planes(ws, j, p, raw1)};
    const int ch[2] = {ch0, ch1};
    float* d_power = (float*)j.out(power, (size_t)2 * nspec * nb * 4, false);
    float2* d_xpol = (float2*)j.out(xpol, (size_t)nspec * nb * 8, false);
    float2* d_bins = p->pcal_tonebins > 0 ? (float2*)j.out(pcal_bins, (size_t)2 * nspec * p->pcal_tonebins * 8, false)
                                          : nullptr;
    float* win = (float*)j.scratch((size_t)(nwin * N * 4));
    float2* X[2] = {(float2*)j.scratch((size_t)(nwin * nb * 8)), (float2*)j.scratch((size_t)(nwin * nb * 8))};
    for (int s = 0; s < 2 && !j.err; s++) {
        const uint8_t* plane = sp[s].planes + (long long)ch[s] * sp[s].bytes_per_sub;
        if ((long long)nspec * p->ffts_per_spectrum * N > sp[s].bytes_per_sub * 4) {
            j.err = set_err(CELLSPE_ERR_ARG, "spectrometer_xpol: spectra need more samples than the recording holds");
            break;
        }
        int rc = map_rc(cs_spec_windows(plane, sp[s].vmask, N, p->overlap, p->ffts_per_spectrum, nspec, p->window, lut,
                                        win, ws.stream), "windows");
        if (!rc) rc = map_rc(cs_rfft_batch(win, X[s], N, nwin, ws.stream), "window FFTs");
        if (!rc && d_bins) {
            // phase-cal of this source alone: the FFT count advances after
            // both sources' FFTs (two sources share it)
            CsSpecArgs a = spec_args(p, sp[s], lut);
            a.planes = plane; a.nsub = 1; a.skip_power = 1;
            a.pcal_sources = 2; a.pcal_source = s;
            a.pcal_bins = d_bins + (size_t)s * nspec * p->pcal_tonebins;
            a.partial = (float*)j.scratch((size_t)cs_spectrometer_scratch_floats(a) * 4);
            if (!j.err) rc = map_rc(cs_spectrometer(a, ws.stream), "phase-cal");
        }
        if (rc) j.err = rc;
    }
    if (!j.err) {
        int rc = map_rc(cs_xpol_reduce(X[0], X[1], N, p->overlap, p->ffts_per_spectrum, nspec, d_power, d_xpol,
                                       ws.stream), "cross spectrum");
        if (rc) j.err = rc;
    }
    return j.finish();
}


// ---------------------------------------------------------------------------
// correlation service: continuous batching over execution streams
// ---------------------------------------------------------------------------
struct SvcJob {
    long long id = 0;
    cellspe_fx_params p{};
    const void* raw = nullptr;
    const double* poly = nullptr;
    void* vis = nullptr;
    long long footprint = 0;
    cudaEvent_t ready = nullptr;      // device buffers complete (legacy stream at submit)
    std::chrono::steady_clock::time_point t_submit, t_start, t_done;
    int status = 0;
    bool large = false;               // runs while no other large job does
    std::string error;                // the worker's message when status != 0
    bool done = false;
};

}  // namespace

struct cellspe_service {
    CopyChain chain;                  // input-copy order of host-buffer jobs
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<std::shared_ptr<SvcJob>> queue;
    std::unordered_map<long long, std::shared_ptr<SvcJob>> jobs;
    std::vector<std::thread> workers;
    std::vector<double> latency_ms, queue_ms;
    long long budget = 0, in_flight = 0, next_id = 1, completed = 0, failed = 0;
    long long priority_samples = 0;   // smaller jobs run on a high-priority stream (<= 0: none)
    int batch_inputs = 0;             // > 0: small jobs of one shape share launches, up to this many inputs
    long long batched_jobs = 0, batched_launches = 0;
    long long large_samples = 0;      // jobs this large run one at a time (<= 0: no limit)
    int large_running = 0;
    int running = 0, max_running = 0;
    bool stop = false;
};

namespace {

// A job that can share launches with others: device buffers, at most 16
// inputs, tensor-core X stage, no delay model, scale, custom levels or
// accumulation.  Jobs of one batch have the same shape.
bool batchable(const SvcJob& q)
{
    const cellspe_fx_params& p = q.p;
    return p.memory == CELLSPE_MEM_DEVICE && !q.poly && p.n_inputs <= 16 && p.x_mode == CELLSPE_X_TC_FP16 &&
           !p.accumulate && !p.custom_levels && !p.channel_scale && !q.large;
}

bool same_shape(const SvcJob& a, const SvcJob& b)
{
    return a.p.fft_points == b.p.fft_points && a.p.n_segments == b.p.n_segments && a.p.levels == b.p.levels &&
           a.p.bytes_per_input == b.p.bytes_per_input && a.p.start_sample == b.p.start_sample;
}

// One stacked job for the batch: the members' inputs back to back (device
// copies), one FX correlation, then each member's triangle gathered out of
// the stacked one.  Per-input F-stage results do not depend on the other
// inputs, and the X stage sums each product over the same segments in the
// same order, so a member's visibilities equal its solo run's.
int run_batch(Workspace& ws, const std::vector<std::shared_ptr<SvcJob>>& batch)
{
    const cellspe_fx_params& p0 = batch[0]->p;
    int S = 0;
    for (auto& m : batch) S += m->p.n_inputs;
    const long long bpi = p0.bytes_per_input, C = p0.fft_points / 2, P = (long long)S * (S + 1) / 2;
    char* d_raw = nullptr;
    float2* d_vis = nullptr;
    cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&d_raw), (size_t)(S * bpi), ws.stream);
    if (e == cudaSuccess) e = cudaMallocAsync(reinterpret_cast<void**>(&d_vis), (size_t)(C * P * 8), ws.stream);
    int rc = e == cudaSuccess ? 0 : cuda_fail(e, "batch buffers");
    long long off = 0;
    for (size_t b = 0; b < batch.size() && !rc; b++) {
        const long long n = (long long)batch[b]->p.n_inputs * bpi;
        e = cudaMemcpyAsync(d_raw + off * bpi, batch[b]->raw, (size_t)n, cudaMemcpyDeviceToDevice, ws.stream);
        if (e != cudaSuccess) rc = cuda_fail(e, "batch input copy");
        off += batch[b]->p.n_inputs;
    }
    if (!rc) {
        cellspe_fx_params sp = p0;
        sp.n_inputs = S;
        sp.vis_order = CELLSPE_VIS_CHANNEL_MAJOR;
        rc = op_fx(ws, &sp, d_raw, nullptr, d_vis, true);
    }
    if (!rc) {
        CsGatherArgs g{};
        g.n = (int)batch.size();
        g.C = (int)C;
        g.P_stacked = P;
        g.src = d_vis;
        int o = 0;
        for (size_t b = 0; b < batch.size(); b++) {
            g.job[b] = {o, batch[b]->p.n_inputs, static_cast<float2*>(batch[b]->vis),
                        batch[b]->p.vis_order == CELLSPE_VIS_BASELINE_MAJOR ? 1 : 0};
            o += batch[b]->p.n_inputs;
        }
        rc = map_rc(cs_vis_gather(g, ws.stream), "batch gather");
        if (!rc) {
            e = cudaStreamSynchronize(ws.stream);
            if (e != cudaSuccess) rc = cuda_fail(e, "batch gather");
        }
    }
    if (d_raw) cudaFreeAsync(d_raw, ws.stream);
    if (d_vis) cudaFreeAsync(d_vis, ws.stream);
    return rc;
}

void service_worker(cellspe_service* sv)
{
    Workspace ws;
    int init = ws.init();
    ws.chain = &sv->chain;
    cs_fstage_allow_timing(false);       // no schedule timing inside a live job
    // small jobs go to a stream of the greatest priority: the block scheduler
    // then dispatches their thread blocks before the waiting blocks of large
    // jobs' kernels, instead of after the whole grid
    cudaStream_t lo = ws.stream, hi = nullptr;
    int least = 0, greatest = 0;
    if (!init && sv->priority_samples > 0 && cudaDeviceGetStreamPriorityRange(&least, &greatest) == cudaSuccess &&
        greatest < least && cudaStreamCreateWithPriority(&hi, cudaStreamNonBlocking, greatest) != cudaSuccess) {
        hi = nullptr;
        cudaGetLastError();
    }
    std::unique_lock<std::mutex> lk(sv->mu);
    for (;;) {
        // admit the oldest job whose device footprint fits next to the jobs
        // already running (a lone job always fits); with a large-job limit,
        // a large job is passed over while another large job runs.
        auto pick = [&]() -> std::deque<std::shared_ptr<SvcJob>>::iterator {
            for (auto it = sv->queue.begin(); it != sv->queue.end(); ++it) {
                const SvcJob& q = **it;
                if (q.large && sv->large_running > 0) continue;
                if (sv->in_flight == 0 || sv->in_flight + q.footprint <= sv->budget) return it;
                return sv->queue.end();          // memory goes to the oldest job that needs it
            }
            return sv->queue.end();
        };
        std::deque<std::shared_ptr<SvcJob>>::iterator at;
        sv->cv_work.wait(lk, [&] { return sv->stop || (at = pick()) != sv->queue.end(); });
        if (sv->stop) break;
        std::shared_ptr<SvcJob> j = *at;
        sv->queue.erase(at);
        // batching: queued jobs of the same shape join a small job (one F-stage
        // and one X-stage launch for all of them)
        std::vector<std::shared_ptr<SvcJob>> batch{j};
        if (sv->batch_inputs > 0 && batchable(*j)) {
            int total = j->p.n_inputs;
            for (auto it = sv->queue.begin(); it != sv->queue.end() && (int)batch.size() < CS_GATHER_MAX;) {
                const SvcJob& q = **it;
                if (batchable(q) && same_shape(q, *j) && total + q.p.n_inputs <= sv->batch_inputs) {
                    total += q.p.n_inputs;
                    batch.push_back(*it);
                    it = sv->queue.erase(it);
                } else {
                    ++it;
                }
            }
        }
        long long footprint = 0;
        for (auto& m : batch) footprint += m->footprint;
        if (j->large) sv->large_running++;
        sv->in_flight += footprint;
        sv->running++;
        sv->max_running = std::max(sv->max_running, sv->running);
        if (batch.size() > 1) {
            sv->batched_jobs += (long long)batch.size();
            sv->batched_launches++;
        }
        lk.unlock();
        sv->cv_work.notify_all();
        const auto t_start = std::chrono::steady_clock::now();
        for (auto& m : batch) m->t_start = t_start;
        int rc = init;
        const long long samples = (long long)j->p.n_inputs * j->p.fft_points * j->p.n_segments;
        ws.stream = (hi && samples < sv->priority_samples) ? hi : lo;
        for (auto& m : batch)
            if (!rc && m->ready) {
                cudaError_t e = cudaStreamWaitEvent(ws.stream, m->ready, 0);
                if (e != cudaSuccess) rc = cuda_fail(e, "service job ordering");
            }
        if (!rc) rc = batch.size() > 1 ? run_batch(ws, batch) : op_fx(ws, &j->p, j->raw, j->poly, j->vis, true);
        ws.stream = lo;
        const auto t_done = std::chrono::steady_clock::now();
        const std::string err = rc ? t_err : std::string();
        lk.lock();
        if (j->large) sv->large_running--;
        sv->in_flight -= footprint;
        sv->running--;
        for (auto& m : batch) {
            if (m->ready) {
                cudaEventDestroy(m->ready);
                m->ready = nullptr;
            }
            m->t_done = t_done;
            m->status = rc;
            if (rc) m->error = err;
            m->done = true;
            if (rc) sv->failed++;
            else {
                sv->completed++;
                sv->latency_ms.push_back(std::chrono::duration<double, std::milli>(m->t_done - m->t_submit).count());
                sv->queue_ms.push_back(std::chrono::duration<double, std::milli>(m->t_start - m->t_submit).count());
            }
        }
        sv->cv_done.notify_all();
        sv->cv_work.notify_all();
    }
    lk.unlock();
    if (hi) cudaStreamSynchronize(hi), cudaStreamDestroy(hi);
    ws.destroy();
}

double percentile(std::vector<double> v, double q)
{
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    double pos = q * (double)(v.size() - 1);
    size_t i = (size_t)pos;
    double f = pos - (double)i;
    return i + 1 < v.size() ? v[i] * (1 - f) + v[i + 1] * f : v[i];
}

// ---------------------------------------------------------------------------
// task runtime
// ---------------------------------------------------------------------------
struct Slot {
    std::thread th;
    std::mutex mu;
    std::condition_variable cv;
    CellDSPTask_t* pending = nullptr;
    bool running = false, done = false, quit = false, has_result = false;
    int result = 0;
    unsigned flags = CDSP_EF_DEFAULT;
    int fft_n = 0;
    std::atomic<int> inject{0};
    Workspace ws;
};

struct Engine {
    std::mutex mu;
    std::condition_variable freecv;
    Slot slots[CELLDSP_MAX_SPE_NR];
    int clients = 0;
    unsigned behaviour = CDSP_BEHAV_DEFAULT;
    int free_waiters = 0;
};

std::mutex g_eng_mu;
Engine* g_eng = nullptr;

struct Vec {
    void* p;
    size_t n;
};
Vec invec(CellDSPTask_t* t, unsigned i) { return {t->inputvector_ptrs[i].p, t->inputvector_lengths[i]}; }
Vec outvec(CellDSPTask_t* t, unsigned i) { return {t->outputvector_ptrs[i].p, t->outputvector_lengths[i]}; }

int complex_op(Slot& s, CellDSPTask_t* t, bool host, int kind)
{
    if (t->num_input_vectors < 2 || t->num_output_vectors < 1) return CELLDSP_TASK_GENERICERROR;
    Vec a = invec(t, 0), b = invec(t, 1), o = outvec(t, 0);
    size_t n = a.n / 8;
    if (b.n < n * 8 || o.n < n * 8) return CELLDSP_TASK_GENERICERROR;
    Job j(s.ws, host);
    const float2* da = (const float2*)j.in(a.p, n * 8);
    const float2* db = (const float2*)j.in(b.p, n * 8);
    float2* dout = (float2*)j.out(o.p, n * 8, kind <= 1);
    if (!j.err) {
        int rc = 0;
        switch (kind) {
            case 0: rc = cs_cmac(da, db, dout, n, 0, s.ws.stream); break;
            case 1: rc = cs_cmac(da, db, dout, n, 1, s.ws.stream); break;
            case 2: rc = cs_cmul(da, db, dout, n, s.ws.stream); break;
            default: rc = cs_cadd(da, db, dout, n, s.ws.stream); break;
        }
        rc = map_rc(rc, "vector op");
        if (rc) j.err = rc;
    }
    return j.finish() ? CELLDSP_TASK_GENERICERROR : CELLDSP_TASK_OK;
}

// CELLDSP_TASK_DIFXPROCESS (exec_difxprocess, cellspe-tasklib-dsp.cpp:609-698):
// in0 nfft complex points, in-place FFT; the band starts at in0 (lower) or
// outputvector_lengths[0] bytes into the FFT output (upper, as the reference
// indexes it); band[i] *= complexfracmult[i] for numchannels points;
// autocorr[i].re += |band[i]|^2 (out2, read-modify-write); out0 <- band.
// The FFT buffer is padded with zeros so that the upper-band window of the
// reference never reads past it.
int difx_op(Slot& s, CellDSPTask_t* t, bool host)
{
    if (t->num_input_vectors < 2 || t->num_output_vectors < 3) return CELLDSP_TASK_GENERICERROR;
    const CellDSPParams_Difx_t& d = t->subcontext.Difx;
    int nfft = (int)d.nfft, nch = (int)d.numchannels;
    Vec in0 = invec(t, 0), in1 = invec(t, 1), o0 = outvec(t, 0), o2 = outvec(t, 2);
    if (!pow2(nfft) || in0.n < (size_t)nfft * 8 || in1.n < (size_t)nch * 8 || o2.n < (size_t)nch * 8)
        return CELLDSP_TASK_GENERICERROR;
    size_t band_off = d.useUpperOrLower ? o0.n : 0;
    size_t pad = (size_t)nfft * 8 + band_off + o0.n + (size_t)nch * 8;
    Job j(s.ws, host);
    const float2* din = (const float2*)j.in(in0.p, (size_t)nfft * 8);
    const float2* dmul = (const float2*)j.in(in1.p, (size_t)nch * 8);
    float2* dacc = (float2*)j.out(o2.p, o2.n, true);
    char* fft = (char*)j.scratch(pad);
    if (!j.err) {
        cudaError_t e = cudaMemsetAsync(fft, 0, pad, s.ws.stream);
        int rc = e == cudaSuccess ? map_rc(cs_cfft_batch(din, (float2*)fft, nfft, 1, s.ws.stream), "difx fft")
                                  : cuda_fail(e, "memset");
        float2* band = (float2*)(fft + band_off);
        if (!rc) rc = map_rc(cs_cmul(dmul, band, band, nch, s.ws.stream), "difx mul");
        if (!rc) rc = map_rc(cs_autocorr_acc(band, dacc, nch, s.ws.stream), "difx autocorr");
        if (!rc) {
            if (host) s.ws.outs.push_back({o0.p, band, o0.n});
            else {
                cudaError_t e2 = cudaMemcpyAsync(o0.p, band, o0.n, cudaMemcpyDeviceToDevice, s.ws.stream);
                if (e2 != cudaSuccess) rc = cuda_fail(e2, "difx copy");
            }
        }
        if (rc) j.err = rc;
    }
    return j.finish() ? CELLDSP_TASK_GENERICERROR : CELLDSP_TASK_OK;
}

int run_task(Slot& s, CellDSPTask_t* t)
{
    const unsigned cmd = t->command & CELLDSP_TASK_CMD_MASK;
    const bool host = !(t->command & CELLDSP_TASK_FLAG_DEVPTR);
    if (s.inject.load() > 0) {
        s.inject--;
        set_err(CELLSPE_ERR_INJECTED, "injected task failure");
        return CELLDSP_TASK_GENERICERROR;
    }
    switch (cmd) {
        case CELLDSP_TASK_NOP:
        case CELLDSP_TASK_IOBENCH:
        case CELLDSP_TASK_RUNALL:
        case CELLDSP_TASK_DMASIMULATION:
            return CELLDSP_TASK_OK;
        case CELLDSP_TASK_IOTEST: {   // do_in_out_test, cellspe-tasklib-dsp.cpp:1121-1131
            if (t->num_output_vectors < 1 || t->outputvector_lengths[0] < 16) return CELLDSP_TASK_GENERICERROR;
            const float v[4] = {0.1f, 2.3f, 4.5f, 6.7f};
            if (host) std::memcpy(t->outputvector_ptrs[0].p, v, sizeof v);
            else if (cudaMemcpy(t->outputvector_ptrs[0].p, v, sizeof v, cudaMemcpyHostToDevice) != cudaSuccess)
                return CELLDSP_TASK_GENERICERROR;
            return CELLDSP_TASK_OK;
        }
        case CELLDSP_TASK_MAC: return complex_op(s, t, host, 0);
        case CELLDSP_TASK_MAC_CONJ: return complex_op(s, t, host, 1);
        case CELLDSP_TASK_MULC: return complex_op(s, t, host, 2);
        case CELLDSP_TASK_ADDC: return complex_op(s, t, host, 3);
        case CELLDSP_TASK_FFT_INIT: {
            int n = (int)t->subcontext.FFT.nfft;
            if (!pow2(n) || n < 16 || n > 16384) return CELLDSP_TASK_GENERICERROR;
            if (!cs_twiddles(2 * n)) return CELLDSP_TASK_GENERICERROR;
            s.fft_n = n;
            return CELLDSP_TASK_OK;
        }
        case CELLDSP_TASK_FFT_FREE:
            s.fft_n = 0;
            return CELLDSP_TASK_OK;
        case CELLDSP_TASK_FFT_EXEC:
        case CELLDSP_TASK_FFT_EXEC_DYN: {
            int n = (int)t->subcontext.FFT.nfft;
            if (cmd == CELLDSP_TASK_FFT_EXEC && n != s.fft_n) return CELLDSP_TASK_GENERICERROR;
            if (t->num_input_vectors < 1 || t->num_output_vectors < 1 || !pow2(n)) return CELLDSP_TASK_GENERICERROR;
            long long batch = t->inputvector_lengths[0] / (8LL * n);
            if (batch < 1 || t->outputvector_lengths[0] < (size_t)batch * n * 8) return CELLDSP_TASK_GENERICERROR;
            return op_fft(s.ws, host, t->inputvector_ptrs[0].p, t->outputvector_ptrs[0].p, n, batch, false)
                       ? CELLDSP_TASK_GENERICERROR : CELLDSP_TASK_OK;
        }
        case CELLDSP_TASK_RFFT: {
            int n = (int)t->subcontext.FFT.nfft;
            if (t->num_input_vectors < 1 || t->num_output_vectors < 1 || !pow2(n)) return CELLDSP_TASK_GENERICERROR;
            long long batch = t->inputvector_lengths[0] / (4LL * n);
            if (batch < 1 || t->outputvector_lengths[0] < (size_t)batch * (n / 2 + 1) * 8) return CELLDSP_TASK_GENERICERROR;
            return op_fft(s.ws, host, t->inputvector_ptrs[0].p, t->outputvector_ptrs[0].p, n, batch, true)
                       ? CELLDSP_TASK_GENERICERROR : CELLDSP_TASK_OK;
        }
        case CELLDSP_TASK_SINCOS:
        case CELLDSP_TASK_SINCOS_NORM: {
            if (t->num_input_vectors < 1 || t->num_output_vectors < 1) return CELLDSP_TASK_GENERICERROR;
            size_t n = t->subcontext.Phase.argcount ? t->subcontext.Phase.argcount : t->inputvector_lengths[0] / 4;
            if (t->inputvector_lengths[0] < n * 4 || t->outputvector_lengths[0] < n * 8) return CELLDSP_TASK_GENERICERROR;
            Job j(s.ws, host);
            const float* din = (const float*)j.in(t->inputvector_ptrs[0].p, n * 4);
            float2* dout = (float2*)j.out(t->outputvector_ptrs[0].p, n * 8, false);
            if (!j.err) {
                int rc = map_rc(cs_sincos(din, dout, n, cmd == CELLDSP_TASK_SINCOS_NORM, s.ws.stream), "sincos");
                if (rc) j.err = rc;
            }
            return j.finish() ? CELLDSP_TASK_GENERICERROR : CELLDSP_TASK_OK;
        }
        case CELLDSP_TASK_SINCOS_GENERTR: {
            if (t->num_output_vectors < 1) return CELLDSP_TASK_GENERICERROR;
            size_t n = t->subcontext.Phase.argcount;
            if (t->outputvector_lengths[0] < n * 8) return CELLDSP_TASK_GENERICERROR;
            Job j(s.ws, host);
            float2* dout = (float2*)j.out(t->outputvector_ptrs[0].p, n * 8, false);
            if (!j.err) {
                int rc = map_rc(cs_sincos_generator(t->subcontext.Phase.phase_start, t->subcontext.Phase.phase_delta,
                                                    dout, n, s.ws.stream), "sincos generator");
                if (rc) j.err = rc;
            }
            return j.finish() ? CELLDSP_TASK_GENERICERROR : CELLDSP_TASK_OK;
        }
        case CELLDSP_TASK_UNPACK: {
            const CellDSPParams_Unpack_t& u = t->subcontext.Unpack;
            long long nsamp = (long long)u.nsamp_lo | ((long long)u.nsamp_hi << 32);
            int nch = (int)u.nchan;
            if (t->num_input_vectors < 1 || t->num_output_vectors < 1 || nch < 1) return CELLDSP_TASK_GENERICERROR;
            const float* custom = (t->num_input_vectors >= 2 && t->inputvector_lengths[1] >= 16 && host)
                                      ? (const float*)t->inputvector_ptrs[1].p : nullptr;
            if ((long long)t->inputvector_lengths[0] * 4 < nsamp * nch) return CELLDSP_TASK_GENERICERROR;
            if (t->num_output_vectors == (unsigned)nch && nch > 1) {
                // one output vector per channel: unpack into the workspace, copy planes
                for (int c = 0; c < nch; c++)
                    if (t->outputvector_lengths[c] < (size_t)nsamp * 4) return CELLDSP_TASK_GENERICERROR;
                std::vector<float> tmp((size_t)nsamp * nch);
                float* dst = tmp.data();
                float* dev = nullptr;
                if (!host) {
                    if (cudaMalloc(&dev, (size_t)nsamp * nch * 4) != cudaSuccess) return CELLDSP_TASK_GENERICERROR;
                    dst = dev;
                }
                int rc = op_unpack(s.ws, host, t->inputvector_ptrs[0].p, nsamp, nch, (int)u.format, custom, dst);
                for (int c = 0; c < nch && !rc; c++) {
                    if (host) std::memcpy(t->outputvector_ptrs[c].p, tmp.data() + (size_t)c * nsamp, (size_t)nsamp * 4);
                    else rc = cudaMemcpy(t->outputvector_ptrs[c].p, dev + (size_t)c * nsamp, (size_t)nsamp * 4,
                                         cudaMemcpyDeviceToDevice) != cudaSuccess;
                }
                if (dev) cudaFree(dev);
                return rc ? CELLDSP_TASK_GENERICERROR : CELLDSP_TASK_OK;
            }
            if (t->outputvector_lengths[0] < (size_t)nsamp * nch * 4) return CELLDSP_TASK_GENERICERROR;
            return op_unpack(s.ws, host, t->inputvector_ptrs[0].p, nsamp, nch, (int)u.format, custom,
                             (float*)t->outputvector_ptrs[0].p) ? CELLDSP_TASK_GENERICERROR : CELLDSP_TASK_OK;
        }
        case CELLDSP_TASK_DIFXPROCESS: return difx_op(s, t, host);
        case CELLDSP_TASK_FX_CORRELATE: {
            if (t->num_input_vectors < 2 || t->num_output_vectors < 1 ||
                t->inputvector_lengths[0] < sizeof(cellspe_fx_params)) return CELLDSP_TASK_GENERICERROR;
            cellspe_fx_params p = *(const cellspe_fx_params*)t->inputvector_ptrs[0].p;
            p.memory = host ? CELLSPE_MEM_HOST : CELLSPE_MEM_DEVICE;
            const double* poly = t->num_input_vectors >= 3 ? (const double*)t->inputvector_ptrs[2].p : nullptr;
            return op_fx(s.ws, &p, t->inputvector_ptrs[1].p, poly, t->outputvector_ptrs[0].p, true)
                       ? CELLDSP_TASK_GENERICERROR : CELLDSP_TASK_OK;
        }
        case CELLDSP_TASK_SPECTROMETER: {
            if (t->num_input_vectors < 2 || t->num_output_vectors < 1 ||
                t->inputvector_lengths[0] < sizeof(cellspe_spec_params)) return CELLDSP_TASK_GENERICERROR;
            cellspe_spec_params p = *(const cellspe_spec_params*)t->inputvector_ptrs[0].p;
            p.memory = host ? CELLSPE_MEM_HOST : CELLSPE_MEM_DEVICE;
            void* bins = t->num_output_vectors >= 2 ? t->outputvector_ptrs[1].p : nullptr;
            void* tones = t->num_output_vectors >= 3 ? t->outputvector_ptrs[2].p : nullptr;
            return op_spectrometer(s.ws, &p, t->inputvector_ptrs[1].p, (float*)t->outputvector_ptrs[0].p, bins, tones)
                       ? CELLDSP_TASK_GENERICERROR : CELLDSP_TASK_OK;
        }
        case CELLDSP_TASK_XMAC: {
            if (t->num_input_vectors < 2 || t->num_output_vectors < 1 ||
                t->inputvector_lengths[0] < sizeof(cellspe_xmac_params)) return CELLDSP_TASK_GENERICERROR;
            cellspe_xmac_params p = *(const cellspe_xmac_params*)t->inputvector_ptrs[0].p;
            return op_xmac(s.ws, host, t->inputvector_ptrs[1].p, p.S, p.C, p.K, t->outputvector_ptrs[0].p, p.accumulate)
                       ? CELLDSP_TASK_GENERICERROR : CELLDSP_TASK_OK;
        }
        default:
            return CELLDSP_TASK_UNKOWNCOMMAND;
    }
}

void worker_main(Slot* s)
{
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
        s->cv.wait(lk, [&] { return s->quit || s->pending; });
        if (s->pending) {
            CellDSPTask_t* t = s->pending;
            s->pending = nullptr;
            s->running = true;
            lk.unlock();
            int code = CELLDSP_TASK_OK;
            int init = s->ws.init();
            for (; t; t = (CellDSPTask_t*)t->next_task.p) {
                unsigned ns = 0;
                if (init) code = CELLDSP_TASK_GENERICERROR;
                else {
                    cudaEventRecord(s->ws.ev0, s->ws.stream);
                    code = run_task(*s, t);
                    cudaEventRecord(s->ws.ev1, s->ws.stream);
                    float ms = 0.f;
                    if (cudaEventSynchronize(s->ws.ev1) == cudaSuccess &&
                        cudaEventElapsedTime(&ms, s->ws.ev0, s->ws.ev1) == cudaSuccess) {
                        double v = (double)ms * 1e6;
                        ns = v >= 4294967295.0 ? 0xFFFFFFFFu : (unsigned)v;
                    }
                }
                t->tick_count = ns;
                t->completed_flag = (unsigned short)code;
                if (code != CELLDSP_TASK_OK)
                    std::cerr << "cellspe task (cmd=" << t->command << ") failed: " << t_err << std::endl;
            }
            lk.lock();
            s->running = false;
            s->done = true;
            s->has_result = true;
            s->result = code;
            s->cv.notify_all();
        }
        if (s->quit && !s->pending) break;
    }
    lk.unlock();
    s->ws.destroy();
}

}  // namespace

int cs_set_error(int code, const char* msg) { return set_err(code, msg ? msg : ""); }
bool cs_pick_levels(int format, const float* custom, float out[4]) { return pick_levels(format, custom, out); }
int cs_spec_check(const cellspe_spec_params* p, const char* who) { return spec_check(p, who); }

// ===========================================================================
// exported: task runtime
// ===========================================================================
extern "C" {

int celldsp_start(void)
{
    std::lock_guard<std::mutex> g(g_eng_mu);
    if (g_eng) {
        std::lock_guard<std::mutex> lk(g_eng->mu);
        g_eng->clients++;
        std::cerr << "celldsp_start: client " << g_eng->clients << " re-uses the running engine" << std::endl;
        return 0;
    }
    if (ensure_device()) {
        std::cerr << "celldsp_start: " << t_err << std::endl;
        return -1;
    }
    g_eng = new Engine();
    g_eng->clients = 1;
    for (auto& s : g_eng->slots) s.th = std::thread(worker_main, &s);
    return 0;
}

int celldsp_stop(void)
{
    std::lock_guard<std::mutex> g(g_eng_mu);
    if (!g_eng) return -1;
    {
        std::lock_guard<std::mutex> lk(g_eng->mu);
        if (--g_eng->clients > 0) {
            std::cerr << "celldsp_stop: other clients still use the engine" << std::endl;
            return 0;
        }
    }
    for (auto& s : g_eng->slots) {
        {
            std::lock_guard<std::mutex> lk(s.mu);
            s.quit = true;
        }
        s.cv.notify_all();
    }
    for (auto& s : g_eng->slots) s.th.join();
    delete g_eng;
    g_eng = nullptr;
    return 0;
}

void celldsp_setBehaviour(unsigned int flags)
{
    if (!g_eng) return;
    std::lock_guard<std::mutex> lk(g_eng->mu);
    g_eng->behaviour = flags;
}

unsigned int celldsp_getBehaviour(void) { return g_eng ? g_eng->behaviour : 0; }

int celldsp_getFreeSPE(void)
{
    if (!g_eng) return -1;
    std::unique_lock<std::mutex> lk(g_eng->mu);
    for (;;) {
        for (int i = 0; i < CELLDSP_MAX_SPE_NR; i++) {
            if (!(g_eng->slots[i].flags & CDSP_EF_RESERVED)) {
                g_eng->slots[i].flags |= CDSP_EF_RESERVED;
                return i;
            }
        }
        if (!(g_eng->behaviour & CDSP_BEHAV_BLOCKING)) return -1;
        g_eng->free_waiters++;
        g_eng->freecv.wait(lk);
        g_eng->free_waiters--;
    }
}

int celldsp_setFreeSPE(int targetSPE)
{
    if (!g_eng || targetSPE < 0 || targetSPE >= CELLDSP_MAX_SPE_NR) return -1;
    std::lock_guard<std::mutex> lk(g_eng->mu);
    Slot& s = g_eng->slots[targetSPE];
    if (s.flags & CDSP_EF_RESERVED) {
        s.flags = CDSP_EF_DEFAULT;
        g_eng->freecv.notify_all();
    } else {
        std::cerr << "warning: celldsp_setFreeSPE(SPE " << targetSPE << ") was already free" << std::endl;
    }
    return 0;
}

int celldsp_startTask(int targetSPE, CellDSPTask_t* task)
{
    if (!g_eng || !task || targetSPE < 0 || targetSPE >= CELLDSP_MAX_SPE_NR) return -1;
    Slot& s = g_eng->slots[targetSPE];
    {
        std::lock_guard<std::mutex> lk(g_eng->mu);
        if (!(s.flags & CDSP_EF_RESERVED)) {
            std::cerr << "celldsp_startTask: slot " << targetSPE << " is not reserved" << std::endl;
            return -1;
        }
    }
    std::lock_guard<std::mutex> lk(s.mu);
    if (s.pending || s.running) {
        std::cerr << "celldsp_startTask: slot " << targetSPE << " is busy" << std::endl;
        return -1;
    }
    for (CellDSPTask_t* t = task; t; t = (CellDSPTask_t*)t->next_task.p) t->completed_flag = CELLDSP_TASK_INCOMPLETE;
    s.pending = task;
    s.done = false;
    s.cv.notify_all();
    return 0;
}

int celldsp_waitTask(int targetSPE)
{
    if (!g_eng || targetSPE < 0 || targetSPE >= CELLDSP_MAX_SPE_NR) return -1;
    Slot& s = g_eng->slots[targetSPE];
    std::unique_lock<std::mutex> lk(s.mu);
    if (!s.pending && !s.running && !s.done) {
        std::cerr << "celldsp_waitTask: no task was started on slot " << targetSPE << std::endl;
        return -1;
    }
    s.cv.wait(lk, [&] { return s.done; });
    s.done = false;
    return s.result;
}

int celldsp_executeTask(CellDSPTask_t* task)
{
    int slot = celldsp_getFreeSPE();
    if (slot == -1) {
        std::cerr << "celldsp_executeTask(cmd=" << (task ? task->command : 0) << ") : could not get any free slot" << std::endl;
        return 1;
    }
    if (celldsp_startTask(slot, task) == -1) {
        celldsp_setFreeSPE(slot);
        return 1;
    }
    int result = celldsp_waitTask(slot);
    celldsp_setFreeSPE(slot);
    if (result != CELLDSP_TASK_OK) {
        std::cerr << "celldsp_executeTask : task returned error code " << result << std::endl;
        return 1;
    }
    return 0;
}

int celldsp_startContinuableTask(CellDSPTask_t* task, int* speID)
{
    *speID = celldsp_getFreeSPE();
    if (*speID == -1) return 1;
    if (celldsp_startTask(*speID, task) == -1) {
        celldsp_setFreeSPE(*speID);
        *speID = -1;
        return 1;
    }
    int result = celldsp_waitTask(*speID);
    if (result != CELLDSP_TASK_OK) {
        celldsp_setFreeSPE(*speID);
        *speID = -1;
        return 1;
    }
    g_eng->slots[*speID].flags |= CDSP_EF_CONTINUABLE;
    return 0;
}

int celldsp_continueTask(CellDSPTask_t* task, int* speID)
{
    if (!speID || *speID < 0) return 1;
    if (celldsp_startTask(*speID, task) == -1) return 1;
    return celldsp_waitTask(*speID) == CELLDSP_TASK_OK ? 0 : 1;
}

int celldsp_stopContinuableTask(int* speID)
{
    if (!speID || *speID < 0) return 1;
    celldsp_setFreeSPE(*speID);
    *speID = -1;
    return 0;
}

// ===========================================================================
// exported: spe* wrappers (cellspe-tasklib-dsp.cpp:94-359)
// ===========================================================================
static void task_init(CellDSPTask_t* t, unsigned cmd)
{
    std::memset(t, 0, sizeof *t);
    t->command = cmd;
}
static void add_in(CellDSPTask_t* t, void* p, size_t n)
{
    t->inputvector_ptrs[t->num_input_vectors].p = p;
    t->inputvector_lengths[t->num_input_vectors++] = (unsigned)n;
}
static void add_out(CellDSPTask_t* t, void* p, size_t n)
{
    t->outputvector_ptrs[t->num_output_vectors].p = p;
    t->outputvector_lengths[t->num_output_vectors++] = (unsigned)n;
}

int speNOP(void)
{
    CellDSPTask_t t;
    task_init(&t, CELLDSP_TASK_NOP);
    return celldsp_executeTask(&t);
}

int speRunAllCheck(void)
{
    CellDSPTask_t t;
    task_init(&t, CELLDSP_TASK_RUNALL);
    return celldsp_executeTask(&t);
}

int speIOCheck(void)
{
    static float output[8] __attribute__((aligned(128)));
    CellDSPTask_t t;
    task_init(&t, CELLDSP_TASK_IOTEST);
    add_out(&t, output, sizeof output);
    int status = celldsp_executeTask(&t);
    std::cout << "speIOCheck wrote back : vect={" << output[0] << "," << output[1] << "," << output[2] << ","
              << output[3] << "}   expected would be {0.1,2.3,4.5,6.7}" << std::endl;
    return status;
}

int speIOSimulation(void)
{
    CellDSPTask_t t;
    task_init(&t, CELLDSP_TASK_DMASIMULATION);
    return celldsp_executeTask(&t);
}

int speIOBench(void* buffer, unsigned int bufbytes, int spes)
{
    (void)buffer; (void)bufbytes; (void)spes;
    CellDSPTask_t t;
    task_init(&t, CELLDSP_TASK_IOBENCH);
    return celldsp_executeTask(&t);
}

int speIOBenchStreamed(void* buffer, unsigned int bufbytes, int spes, int stream_length)
{
    (void)stream_length;
    return speIOBench(buffer, bufbytes, spes);
}

int speAddProduct_32fc(fc32* src, fc32* src2, fc32* accumulator, int length)
{
    CellDSPTask_t t;
    task_init(&t, CELLDSP_TASK_MAC);
    add_in(&t, src, (size_t)length * sizeof(fc32));
    add_in(&t, src2, (size_t)length * sizeof(fc32));
    add_out(&t, accumulator, (size_t)length * sizeof(fc32));
    return celldsp_executeTask(&t);
}

int speFFT_init(int fft_len, int* speID)
{
    CellDSPTask_t t;
    task_init(&t, CELLDSP_TASK_FFT_INIT);
    t.subcontext.FFT.nfft = (unsigned)fft_len;
    return celldsp_startContinuableTask(&t, speID);
}

int speFFT_exec(void* in, void* out, int fft_len, int* speID)
{
    CellDSPTask_t t;
    task_init(&t, CELLDSP_TASK_FFT_EXEC);
    add_in(&t, in, (size_t)fft_len * sizeof(fc32));
    add_out(&t, out, (size_t)fft_len * sizeof(fc32));
    t.subcontext.FFT.nfft = (unsigned)fft_len;
    return celldsp_continueTask(&t, speID);
}

int speFFT_destroy(int* speID)
{
    CellDSPTask_t t;
    task_init(&t, CELLDSP_TASK_FFT_FREE);
    int status = celldsp_continueTask(&t, speID);
    celldsp_stopContinuableTask(speID);
    return status;
}

int speFFT_singleexec(void* in, void* out, int fft_len)
{
    CellDSPTask_t t;
    task_init(&t, CELLDSP_TASK_FFT_EXEC_DYN);
    add_in(&t, in, (size_t)fft_len * sizeof(fc32));
    add_out(&t, out, (size_t)fft_len * sizeof(fc32));
    t.subcontext.FFT.nfft = (unsigned)fft_len;
    return celldsp_executeTask(&t);
}

int speSinCosGenerator(float startphase, float increment, fc32* cos_sin_out, int numiter)
{
    CellDSPTask_t t;
    task_init(&t, CELLDSP_TASK_SINCOS_GENERTR);
    add_out(&t, cos_sin_out, (size_t)numiter * sizeof(cf32));
    t.subcontext.Phase.argcount = (unsigned)numiter;
    t.subcontext.Phase.phase_start = startphase;
    t.subcontext.Phase.phase_delta = increment;
    return celldsp_executeTask(&t);
}

int speSinCosAccurate(float* argument, cf32* cos_sin_out, int argumentcount)
{
    CellDSPTask_t t;
    task_init(&t, CELLDSP_TASK_SINCOS);
    add_in(&t, argument, (size_t)argumentcount * sizeof(float));
    add_out(&t, cos_sin_out, (size_t)argumentcount * sizeof(cf32));
    t.subcontext.Phase.argcount = (unsigned)argumentcount;
    return celldsp_executeTask(&t);
}

int speSinCosAccurateNorm(float* normalizedargument, cf32* cos_sin_out, int argumentcount)
{
    CellDSPTask_t t;
    task_init(&t, CELLDSP_TASK_SINCOS_NORM);
    add_in(&t, normalizedargument, (size_t)argumentcount * sizeof(float));
    add_out(&t, cos_sin_out, (size_t)argumentcount * sizeof(cf32));
    t.subcontext.Phase.argcount = (unsigned)argumentcount;
    return celldsp_executeTask(&t);
}

int speDIFX_process(void* sincosrotdone, void* complexfracmult, void* fftoutJ, void* conjfftoutJ, void* autocorr,
                    int nfft, int twicenumchannels, int useUpperOrLower)
{
    size_t dual_array_len = (size_t)twicenumchannels * sizeof(cf32);
    size_t normal_array_len = (size_t)(twicenumchannels / 2 + 1 + 3) * sizeof(cf32);
    CellDSPTask_t t;
    task_init(&t, CELLDSP_TASK_DIFXPROCESS);
    add_in(&t, sincosrotdone, dual_array_len);
    add_in(&t, complexfracmult, normal_array_len);
    add_out(&t, fftoutJ, normal_array_len);
    add_out(&t, conjfftoutJ, normal_array_len);
    add_out(&t, autocorr, normal_array_len);
    t.subcontext.Difx.nfft = (unsigned)nfft;
    t.subcontext.Difx.useUpperOrLower = (unsigned)useUpperOrLower;
    t.subcontext.Difx.twicenumchannels = (unsigned)twicenumchannels;
    t.subcontext.Difx.numchannels = (unsigned)(twicenumchannels / 2);
    return celldsp_executeTask(&t);
}

// ===========================================================================
// exported: direct engine entry points
// ===========================================================================
const char* cellspe_last_error(void) { return t_err.c_str(); }

long long cellspe_kernel_launches(void) { return cs_launch_count(); }

int cellspe_last_stage_times(float* ms, int n)
{
    if (!ms || n < 0) return CELLSPE_ERR_ARG;
    for (int i = 0; i < n && i < 4; i++) ms[i] = t_stage_ms[i];
    return 0;
}

int cellspe_device_count(void)
{
    int n = 0;
    return cudaGetDeviceCount(&n) == cudaSuccess ? n : 0;
}

int cellspe_set_hbm_budget(long long bytes)
{
    if (bytes < 0) return CELLSPE_ERR_ARG;
    g_budget = bytes;
    return 0;
}

long long cellspe_get_hbm_budget(void) { return budget_bytes(); }

void* cellspe_host_alloc(size_t bytes)
{
    if (ensure_device()) return nullptr;
    void* p = nullptr;
    return cudaHostAlloc(&p, bytes, cudaHostAllocDefault) == cudaSuccess ? p : nullptr;
}

void cellspe_host_free(void* p)
{
    if (p) cudaFreeHost(p);
}

void* cellspe_device_alloc(size_t bytes)
{
    if (ensure_device()) return nullptr;
    void* p = nullptr;
    return cudaMalloc(&p, bytes) == cudaSuccess ? p : nullptr;
}

void cellspe_device_free(void* p)
{
    if (p) cudaFree(p);
}

int cellspe_memcpy(void* dst, const void* src, size_t bytes, int kind)
{
    if (ensure_device()) return CELLSPE_ERR_CUDA;
    cudaMemcpyKind k = kind == 1 ? cudaMemcpyHostToDevice : kind == 2 ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    cudaError_t e = cudaMemcpy(dst, src, bytes, k);
    return e == cudaSuccess ? 0 : cuda_fail(e, "cellspe_memcpy");
}

int cellspe_debug_inject_failure(int slot, int count)
{
    if (slot < 0) {
        g_inject_direct = count;
        return 0;
    }
    if (!g_eng || slot >= CELLDSP_MAX_SPE_NR) return CELLSPE_ERR_ARG;
    g_eng->slots[slot].inject = count;
    return 0;
}

static int direct_gate()
{
    if (g_inject_direct.load() > 0) {
        g_inject_direct--;
        return set_err(CELLSPE_ERR_INJECTED, "injected failure");
    }
    return 0;
}

// Synchronous direct calls: the thread's workspace, its stream ordered after
// the legacy default stream.  Calls on a caller's stream (the async entry
// point, which may run under stream capture) take the workspace only.
#define DIRECT_WORKSPACE                        \
    int _g = direct_gate();                     \
    if (_g) return _g;                          \
    int _rc = 0;                                \
    Workspace* ws = thread_ws(&_rc);            \
    if (!ws) return _rc;
#define DIRECT_PROLOGUE                         \
    DIRECT_WORKSPACE                            \
    if ((_rc = ws->after_legacy_stream())) return _rc;

int cellspe_unpack2bit(const void* raw, long long nsamp, int nchan, int format, const float* custom_levels, float* out,
                       int memory)
{
    DIRECT_PROLOGUE
    return op_unpack(*ws, memory == CELLSPE_MEM_HOST, raw, nsamp, nchan, format, custom_levels, out);
}

int cellspe_fft_c2c(const void* in, void* out, int n, long long batch, int memory)
{
    DIRECT_PROLOGUE
    return op_fft(*ws, memory == CELLSPE_MEM_HOST, in, out, n, batch, false);
}

int cellspe_fft_r2c(const float* in, void* out, int n, long long batch, int memory)
{
    DIRECT_PROLOGUE
    return op_fft(*ws, memory == CELLSPE_MEM_HOST, in, out, n, batch, true);
}

int cellspe_fft_r2c_perm(const float* in, float* out, int n, long long batch, int memory)
{
    DIRECT_PROLOGUE
    return op_fft_perm(*ws, memory == CELLSPE_MEM_HOST, in, out, n, batch);
}

int cellspe_accumulate_f32(float* acc, const float* add, long long n, int memory)
{
    DIRECT_PROLOGUE
    if (!acc || !add || n < 0) return set_err(CELLSPE_ERR_ARG, "accumulate_f32: bad arguments");
    if (n == 0) return 0;
    const bool host = memory == CELLSPE_MEM_HOST;
    Job j(*ws, host);
    const float* d_add = (const float*)j.in(add, (size_t)n * 4);
    float* d_acc = (float*)j.out(acc, (size_t)n * 4, true);
    if (!j.err) {
        int rc = map_rc(cs_fadd(d_add, d_acc, n, ws->stream), "accumulate_f32");
        if (rc) j.err = rc;
    }
    return j.finish();
}

int cellspe_vis_lags(const void* vis, void* lags, long long n_products, int n_channels, double scale, int memory)
{
    DIRECT_PROLOGUE
    if (!vis || !lags || n_products <= 0 || !pow2(n_channels) || n_channels < 16 || n_channels > 16384)
        return set_err(CELLSPE_ERR_ARG, "vis_lags: need products > 0 and n_channels a power of two in [16, 16384]");
    const bool host = memory == CELLSPE_MEM_HOST;
    const size_t bytes = (size_t)n_products * n_channels * 8;
    Job j(*ws, host);
    const float2* d_in = (const float2*)j.in(vis, bytes);
    float2* d_out = (float2*)j.out(lags, bytes, false);
    if (!j.err) {
        int rc = map_rc(cs_cfft_inverse_batch(d_in, d_out, n_channels, n_products, (float)scale, ws->stream), "vis_lags");
        if (rc) j.err = rc;
    }
    return j.finish();
}

int cellspe_xmac(const void* spectra, int S, int C, int K, void* vis, int accumulate, int memory)
{
    DIRECT_PROLOGUE
    return op_xmac(*ws, memory == CELLSPE_MEM_HOST, spectra, S, C, K, vis, accumulate);
}

int cellspe_xmac_f16(const void* spectra_f16, int S, int C, int K, void* vis, int accumulate, int memory)
{
    DIRECT_PROLOGUE
    return op_xmac_f16(*ws, memory == CELLSPE_MEM_HOST, spectra_f16, S, C, K, vis, accumulate);
}

int cellspe_xmac_i8(const void* planes_i8, const float* scale, int S, int C, int K, void* vis, int accumulate,
                    int memory)
{
    DIRECT_PROLOGUE
    return op_xmac_i8(*ws, memory == CELLSPE_MEM_HOST, planes_i8, scale, S, C, K, vis, accumulate);
}

int cellspe_fx_correlate(const cellspe_fx_params* p, const void* raw, const double* delay_poly, void* vis)
{
    DIRECT_PROLOGUE
    return op_fx(*ws, p, raw, delay_poly, vis, true);
}

long long cellspe_fx_workspace_bytes(const cellspe_fx_params* p) { return p ? fx_bytes(p, true) : -1; }

int cellspe_fx_correlate_async(const cellspe_fx_params* p, const void* raw, const double* delay_poly, void* vis,
                               void* stream)
{
    DIRECT_WORKSPACE
    if (!p || p->memory != CELLSPE_MEM_DEVICE) return set_err(CELLSPE_ERR_ARG, "fx async: device memory only");
    cudaStream_t saved = ws->stream;
    ws->stream = (cudaStream_t)stream;
    ws->arena.rewind();
    int rc = op_fx(*ws, p, raw, delay_poly, vis, false);
    ws->stream = saved;
    return rc;
}

int cellspe_release_workspace(void)
{
    if (t_ws) {
        t_ws->destroy();
        t_ws.reset();
    }
    return 0;
}


// ===========================================================================
// exported: correlation service
// ===========================================================================
cellspe_service* cellspe_service_create(const cellspe_service_config* cfg)
{
    if (ensure_device()) return nullptr;
    auto* sv = new cellspe_service();
    long long b = (cfg && cfg->hbm_budget_bytes > 0) ? cfg->hbm_budget_bytes : (long long)(0.8 * (double)budget_bytes() / 0.9);
    sv->budget = b;
    if (cudaEventCreateWithFlags(&sv->chain.in_done, cudaEventDisableTiming) != cudaSuccess) {
        delete sv;
        cuda_fail(cudaGetLastError(), "service setup");
        return nullptr;
    }
    int n = (cfg && cfg->max_streams > 0) ? cfg->max_streams : 2;
    sv->priority_samples = !cfg || cfg->priority_samples == 0 ? (1LL << 24) : cfg->priority_samples;
    sv->large_samples = cfg ? cfg->large_samples : 0;
    // batching is on by default (64 inputs); a negative batch_inputs turns it off
    sv->batch_inputs = !cfg || cfg->batch_inputs == 0 ? 64 : std::max(0, std::min(cfg->batch_inputs, 128));
    for (int i = 0; i < n; i++) sv->workers.emplace_back(service_worker, sv);
    return sv;
}

int cellspe_service_submit(cellspe_service* sv, const cellspe_fx_params* p, const void* raw, const double* delay_poly,
                           void* vis, long long* job_id)
{
    if (!sv || !p || !raw || !vis || !job_id) return set_err(CELLSPE_ERR_ARG, "service_submit: null argument");
    auto j = std::make_shared<SvcJob>();
    j->p = *p;
    j->raw = raw;
    j->poly = delay_poly;
    j->vis = vis;
    j->footprint = fx_bytes(p, delay_poly != nullptr);
    j->large = sv->large_samples > 0 && (long long)p->n_inputs * p->fft_points * p->n_segments >= sv->large_samples;
    if (j->footprint > sv->budget)
        return set_err(CELLSPE_ERR_NOMEM, "service_submit: job footprint exceeds the service HBM budget");
    j->t_submit = std::chrono::steady_clock::now();
    // the job's buffers may be filled by work the caller issued before submit:
    // the worker's stream waits for the legacy default stream as it was now
    if (p->memory == CELLSPE_MEM_DEVICE) {
        cudaError_t e = cudaEventCreateWithFlags(&j->ready, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventRecord(j->ready, cudaStreamLegacy);
        if (e != cudaSuccess) {
            if (j->ready) cudaEventDestroy(j->ready);
            return cuda_fail(e, "service_submit");
        }
    }
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        j->id = sv->next_id++;
        sv->jobs[j->id] = j;
        sv->queue.push_back(j);
    }
    sv->cv_work.notify_all();
    *job_id = j->id;
    return 0;
}

int cellspe_service_wait(cellspe_service* sv, long long job_id, double* latency_ms)
{
    if (!sv) return set_err(CELLSPE_ERR_ARG, "service_wait: null service");
    std::unique_lock<std::mutex> lk(sv->mu);
    auto it = sv->jobs.find(job_id);
    if (it == sv->jobs.end()) return set_err(CELLSPE_ERR_ARG, "service_wait: unknown job id");
    std::shared_ptr<SvcJob> j = it->second;
    sv->cv_done.wait(lk, [&] { return j->done; });
    sv->jobs.erase(job_id);
    if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(j->t_done - j->t_submit).count();
    if (j->status) return set_err(j->status, "service job " + std::to_string(job_id) + ": " + j->error);
    return 0;
}

int cellspe_service_get_stats(cellspe_service* sv, cellspe_service_stats* out)
{
    if (!sv || !out) return CELLSPE_ERR_ARG;
    std::lock_guard<std::mutex> lk(sv->mu);
    out->completed = sv->completed;
    out->failed = sv->failed;
    out->queued = (long long)sv->queue.size();
    out->running = sv->running;
    out->max_running = sv->max_running;
    out->p50_ms = percentile(sv->latency_ms, 0.50);
    out->p99_ms = percentile(sv->latency_ms, 0.99);
    out->p99_queue_ms = percentile(sv->queue_ms, 0.99);
    out->budget_bytes = sv->budget;
    out->batched_jobs = sv->batched_jobs;
    out->batched_launches = sv->batched_launches;
    return 0;
}

void cellspe_service_destroy(cellspe_service* sv)
{
    if (!sv) return;
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        sv->stop = true;
    }
    sv->cv_work.notify_all();
    for (auto& t : sv->workers) t.join();
    for (auto& j : sv->queue)              // never started
        if (j->ready) cudaEventDestroy(j->ready), j->ready = nullptr;
    if (sv->chain.in_done) cudaEventDestroy(sv->chain.in_done);
    delete sv;
}

int cellspe_spectrometer(const cellspe_spec_params* p, const void* raw, float* power, void* pcal_bins, void* pcal_tones)
{
    DIRECT_PROLOGUE
    return op_spectrometer(*ws, p, raw, power, pcal_bins, pcal_tones);
}

long long cellspe_spectrometer_workspace_bytes(const cellspe_spec_params* p) { return p ? spec_bytes(p) : -1; }

int cellspe_spectrometer_xpol(const cellspe_spec_params* p, const void* raw0, const void* raw1, int channel0,
                              int channel1, float* power, void* xpol, void* pcal_bins)
{
    DIRECT_PROLOGUE
    return op_spectrometer_xpol(*ws, p, raw0, raw1, channel0, channel1, power, xpol, pcal_bins);
}

int cellspe_mark5b_decode(const void* framed, long long bytes, int nchan, long long nsamp, float* out, int memory,
                          cellspe_mark5b_info* info)
{
    DIRECT_PROLOGUE
    return op_mark5b_decode(*ws, memory == CELLSPE_MEM_HOST, framed, bytes, nchan, nsamp, out, info);
}

int cellspe_mark5b_deframe(const void* framed, long long bytes, int nchan, long long frames, void* payload,
                           unsigned int* valid_mask, int memory, cellspe_mark5b_info* info)
{
    DIRECT_PROLOGUE
    return op_mark5b_deframe(*ws, memory == CELLSPE_MEM_HOST, framed, bytes, nchan, frames, payload, valid_mask, info);
}

int cellspe_vdif_decode(const void* framed, long long bytes, int nchan, int mbps, long long nsamp, float* out,
                        int memory, cellspe_vdif_info* info)
{
    DIRECT_PROLOGUE
    return op_vdif_decode(*ws, memory == CELLSPE_MEM_HOST, framed, bytes, nchan, mbps, nsamp, out, info);
}

int cellspe_vdif_deframe(const void* framed, long long bytes, int nchan, int mbps, long long frames, void* payload,
                         unsigned int* valid_mask, int memory, cellspe_vdif_info* info)
{
    DIRECT_PROLOGUE
    return op_vdif_deframe(*ws, memory == CELLSPE_MEM_HOST, framed, bytes, nchan, mbps, frames, payload, valid_mask,
                           info);
}

}  // extern "C"
