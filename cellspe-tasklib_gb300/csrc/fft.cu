// K-b: batched forward FFTs for the task API.
//
// cs_cfft_batch replaces _fft_1d_r2 / exec_FFT / exec_FFT_dyn
// (minicorrelator/fft_1d_r2_modified.h:81-534, cellspe-tasklib-dsp.cpp:
// 519-602): complex forward transform, interleaved {re, im}, unscaled.
// cs_rfft_batch replaces genericFFTexec_R (architecture.h:563-578, FFTW r2c
// layout: N/2+1 bins).  Both run CtaFft<M> groups (M/16 threads per
// transform, several transforms per CTA).  Twiddle tables are computed once
// per size in FP64 on the host, rounded to FP32 and kept on the device.
#include "common.cuh"
#include "kernels.h"

#include <atomic>
#include <cmath>
#include <map>
#include <mutex>
#include <vector>

namespace {
std::atomic<long long> g_launches{0};
std::mutex g_tw_mu;
std::map<std::pair<int, int>, float2*> g_tw;   // (device, n) -> table
}  // namespace

long long cs_launch_count() { return g_launches.load(); }
void cs_count_launches(int n) { g_launches += n; }

// The attribute is per function and shared by every thread: two host threads
// launching one kernel with different shared-memory sizes could lower it
// under each other's launch.  It only ever grows here (per device), under a lock.
cudaError_t cs_smem_at_least(const void* fn, int bytes)
{
    static std::mutex mu;
    static std::map<std::pair<int, const void*>, int> cur;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(mu);
    int& v = cur[{dev, fn}];
    if (bytes <= v) return cudaSuccess;
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess) v = bytes;
    return e;
}

const float2* cs_twiddles(int n)
{
    if (n <= 0 || (n & (n - 1))) return nullptr;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    std::lock_guard<std::mutex> lk(g_tw_mu);
    auto it = g_tw.find({dev, n});
    if (it != g_tw.end()) return it->second;
    std::vector<float2> h(n);
    for (int m = 0; m < n; m++) {
        double a = -2.0 * M_PI * (double)m / (double)n;
        h[m] = make_float2((float)std::cos(a), (float)std::sin(a));
    }
    float2* d = nullptr;
    if (cudaMalloc(&d, sizeof(float2) * n) != cudaSuccess) return nullptr;
    if (cudaMemcpy(d, h.data(), sizeof(float2) * n, cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(d);
        return nullptr;
    }
    g_tw[{dev, n}] = d;
    return d;
}

// IPP "Perm" packing of real-FFT bins (ippsDFTFwd_RToPerm_32f, read back by
// TaskCoreIPP::doMaths, TaskCoreIPP.cpp:430, 438-439): each row of n floats is
// [R0, R_{n/2}, Re 1, Im 1, ..., Re n/2-1, Im n/2-1], i.e. the n/2+1 complex
// bins with the (zero) imaginary part of bin 0 replaced by the real Nyquist
// bin and the Nyquist bin dropped.  bins [batch][n/2+1], out [batch][n].
__global__ void k_perm_pack(const float2* __restrict__ bins, float* __restrict__ out, int n, int64_t batch)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;     // float2 slot of the output
    const int half = n / 2;
    if (i >= batch * half) return;
    const int64_t row = i / half;
    const int k = (int)(i - row * half);
    const float2* b = bins + row * (half + 1);
    float2 v = b[k];
    if (k == 0) v.y = b[half].x;
    reinterpret_cast<float2*>(out + row * n)[k] = v;
}

int cs_perm_pack(const float2* bins, float* out, int n, int64_t batch, cudaStream_t st)
{
    if (n < 2 || (n & 1) || batch < 0) return CS_ERR_ARG;
    const int64_t total = batch * (n / 2);
    if (total == 0) return 0;
    k_perm_pack<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(bins, out, n, batch), cs_count_launches(1);
    return (int)cudaGetLastError();
}

void cs_free_twiddles()
{
    std::lock_guard<std::mutex> lk(g_tw_mu);
    int cur = 0;
    cudaGetDevice(&cur);
    for (auto& kv : g_tw) {
        cudaSetDevice(kv.first.first);
        cudaFree(kv.second);
    }
    cudaSetDevice(cur);
    g_tw.clear();
}

namespace {

template <int M> struct BCfg {
    static constexpr int T = M / 16;
    static constexpr int GROUPS = (T >= 128) ? 1 : 128 / T;
    static constexpr int NT = T * GROUPS;
};

// All groups of a CTA advance in lockstep (whole-CTA barriers); groups past
// the end of the batch still take part in the barriers but touch no memory.
// INV: backward transform e^{+2 pi i nk/M} (complex only), computed as
// conj(FFT(conj(x))), with the outputs multiplied by `scale`.
template <int M, bool REAL, bool INV>
__global__ void __launch_bounds__(BCfg<M>::NT) k_fft_batch(const void* __restrict__ in, float2* __restrict__ out,
                                                          int64_t batch, const float2* __restrict__ tw, float scale)
{
    using C = BCfg<M>;
    constexpr int T = C::T;
    extern __shared__ __align__(16) unsigned char smem[];
    const int g = threadIdx.x / T, t = threadIdx.x % T;
    float2* fb = reinterpret_cast<float2*>(smem) + g * fpad_size(M);
    const int64_t b = (int64_t)blockIdx.x * C::GROUPS + g;
    const bool valid = b < batch;
    float2 v[16];
#pragma unroll
    for (int r = 0; r < 16; r++) {
        int n = t + r * T;
        if (!valid) v[r] = make_float2(0.f, 0.f);
        else if (REAL) v[r] = __ldg(reinterpret_cast<const float2*>(in) + b * M + n);  // {x[2n], x[2n+1]}
        else v[r] = __ldg(reinterpret_cast<const float2*>(in) + b * M + n);
        if (INV) v[r].y = -v[r].y;
    }
    auto bar = [] { __syncthreads(); };
    // REAL: the M-point transform of pairs uses the 2M-point table (stride 2);
    // complex: the M-point table is the 2M table at stride 2 as well.
    CtaFft<M, (M >= 2048)>::run(fb, t, v, tw, 2, bar);
    if (!valid) return;
    if constexpr (!REAL) {
#pragma unroll
        for (int r = 0; r < 16; r++) {
            float2 z = fb[fpad(t + r * T)];
            if (INV) z = make_float2(z.x * scale, -z.y * scale);
            out[b * M + t + r * T] = z;
        }
    } else {
        float2* o = out + b * (M + 1);
        for (int kk = t; kk <= M / 2; kk += T) {
            float2 Xk, Xm;
            r2c_pair(fb[fpad(kk)], fb[fpad((M - kk) & (M - 1))], twiddle(tw, kk), Xk, Xm);
            if (kk == 0) {
                o[0] = make_float2(Xk.x, 0.f);
                o[M] = make_float2(Xm.x, 0.f);
            } else {
                o[kk] = Xk;
                if (kk != M / 2) o[M - kk] = Xm;
            }
        }
    }
}

template <int M, bool REAL, bool INV>
int launch_batch(const void* in, float2* out, int64_t batch, float scale, cudaStream_t st)
{
    using C = BCfg<M>;
    const float2* tw = cs_twiddles(2 * M);
    if (!tw) return CS_ERR_ARG;
    size_t smem = (size_t)C::GROUPS * fpad_size(M) * sizeof(float2);
    auto kern = k_fft_batch<M, REAL, INV>;
    CS_CUDA_TRY(cs_smem_at_least(reinterpret_cast<const void*>(kern), (int)smem));
    int64_t blocks = (batch + C::GROUPS - 1) / C::GROUPS;
    kern<<<(unsigned)blocks, C::NT, smem, st>>>(in, out, batch, tw, scale), cs_count_launches(1);
    return (int)cudaGetLastError();
}

template <bool REAL, bool INV>
int dispatch(const void* in, float2* out, int m, int64_t batch, float scale, cudaStream_t st)
{
    switch (m) {
        case 16: return launch_batch<16, REAL, INV>(in, out, batch, scale, st);
        case 32: return launch_batch<32, REAL, INV>(in, out, batch, scale, st);
        case 64: return launch_batch<64, REAL, INV>(in, out, batch, scale, st);
        case 128: return launch_batch<128, REAL, INV>(in, out, batch, scale, st);
        case 256: return launch_batch<256, REAL, INV>(in, out, batch, scale, st);
        case 512: return launch_batch<512, REAL, INV>(in, out, batch, scale, st);
        case 1024: return launch_batch<1024, REAL, INV>(in, out, batch, scale, st);
        case 2048: return launch_batch<2048, REAL, INV>(in, out, batch, scale, st);
        case 4096: return launch_batch<4096, REAL, INV>(in, out, batch, scale, st);
        case 8192: return launch_batch<8192, REAL, INV>(in, out, batch, scale, st);
        case 16384: return launch_batch<16384, REAL, INV>(in, out, batch, scale, st);
        default: return CS_ERR_UNSUPPORTED;
    }
}
}  // namespace

int cs_cfft_batch(const float2* in, float2* out, int n, int64_t batch, cudaStream_t st)
{
    if (!in || !out || batch < 0) return CS_ERR_ARG;
    if (batch == 0) return 0;
    return dispatch<false, false>(in, out, n, batch, 1.f, st);
}

int cs_cfft_inverse_batch(const float2* in, float2* out, int n, int64_t batch, float scale, cudaStream_t st)
{
    if (!in || !out || batch < 0) return CS_ERR_ARG;
    if (batch == 0) return 0;
    return dispatch<false, true>(in, out, n, batch, scale, st);
}

int cs_rfft_batch(const float* in, float2* out, int n, int64_t batch, cudaStream_t st)
{
    if (!in || !out || batch < 0 || (n & 1)) return CS_ERR_ARG;
    if ((uintptr_t)in % 8) return CS_ERR_ARG;
    if (batch == 0) return 0;
    return dispatch<true, false>(in, out, n / 2, batch, 1.f, st);
}
