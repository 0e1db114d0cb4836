// Cross-polarisation spectra: two sources and their cross spectrum, as
// TaskCoreIPP::doMaths computes them with num_sources = 2, num_xpols = 1
// (spectrometer/src/IA-32/TaskCoreIPP.cpp:394-513).
//
// The overlapped windows of both sources are unpacked and windowed into a
// batch (k_spec_windows), transformed by the batched real FFT, and reduced per
// bin over the windows of each spectrum in window order (k_xpol_reduce):
//   auto_s[k] += |X_s[k]|^2           (DC and Nyquist: Re^2, :437-447)
//   xpol[k]   += X_0[k] conj(X_1[k])  (bins 1..N/2-1, :476-479)
//   xpol[0]    = sum Re X_0[0] Re X_1[0],  xpol[N/2] likewise, Im = 0 (:481-485)
// all scaled by 1/core_overlapped_ffts (:491-499).  The products and sums
// use explicit round-to-nearest operations (no fused multiply-add), the
// arithmetic of the CPU code.
#include "common.cuh"
#include "kernels.h"

namespace {

CS_DEV float lut4(const float (&l)[4], unsigned c)
{
    const float lo = (c & 1u) ? l[1] : l[0], hi = (c & 1u) ? l[3] : l[2];
    return (c & 2u) ? hi : lo;
}

// thread per (window, 16-sample word): window w = s * novl + j starts at
// sample s * K * N + j * hop of the plane (a multiple of 16)
__global__ void k_spec_windows(const uint32_t* __restrict__ plane, const uint32_t* __restrict__ vmask, int N, int hop,
                               int novl, int64_t samp_per_spec, int64_t nwin, const float* __restrict__ win,
                               float l0, float l1, float l2, float l3, float* __restrict__ out)
{
    const int wpw = N / 16;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nwin * wpw) return;
    const int64_t w = t / wpw;
    const int wi = (int)(t - w * wpw);
    const int64_t s = w / novl, j = w - s * novl;
    const int64_t word = (s * samp_per_spec + j * hop) / 16 + wi;
    const uint32_t bits = __ldg(plane + word);
    const uint32_t valid = vmask ? __ldg(vmask + (word >> 1)) >> ((word & 1) * 16) : 0xffffu;
    const float lut[4] = {l0, l1, l2, l3};
    float v[16];
#pragma unroll
    for (int q = 0; q < 16; q++) {
        const float x = ((valid >> q) & 1u) ? lut4(lut, (bits >> (2 * q)) & 3u) : 0.f;
        v[q] = __fmul_rn(__ldg(win + 16 * wi + q), x);
    }
    float4* o = reinterpret_cast<float4*>(out + w * N + 16 * wi);
#pragma unroll
    for (int q = 0; q < 4; q++) o[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
}

// thread per (spectrum, bin): windows of the spectrum in order
__global__ void k_xpol_reduce(const float2* __restrict__ X0, const float2* __restrict__ X1, int nspec, int novl,
                              int nb, float scale, float* __restrict__ p0, float* __restrict__ p1,
                              float2* __restrict__ xp)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)nspec * nb) return;
    const int s = (int)(t / nb), k = (int)(t - (int64_t)s * nb);
    const bool edge = (k == 0 || k == nb - 1);
    float a0 = 0.f, a1 = 0.f, xr = 0.f, xi = 0.f;
    for (int j = 0; j < novl; j++) {
        const int64_t i = ((int64_t)s * novl + j) * nb + k;
        const float2 u = X0[i], v = X1[i];
        if (edge) {
            a0 = __fadd_rn(a0, __fmul_rn(u.x, u.x));
            a1 = __fadd_rn(a1, __fmul_rn(v.x, v.x));
            xr = __fadd_rn(xr, __fmul_rn(u.x, v.x));
        } else {
            a0 = __fadd_rn(a0, __fadd_rn(__fmul_rn(u.x, u.x), __fmul_rn(u.y, u.y)));
            a1 = __fadd_rn(a1, __fadd_rn(__fmul_rn(v.x, v.x), __fmul_rn(v.y, v.y)));
            // u conj(v): (u.x v.x + u.y v.y) + i (u.y v.x - u.x v.y)
            xr = __fadd_rn(xr, __fadd_rn(__fmul_rn(u.x, v.x), __fmul_rn(u.y, v.y)));
            xi = __fadd_rn(xi, __fsub_rn(__fmul_rn(u.y, v.x), __fmul_rn(u.x, v.y)));
        }
    }
    p0[t] = __fmul_rn(a0, scale);
    p1[t] = __fmul_rn(a1, scale);
    xp[t] = make_float2(__fmul_rn(xr, scale), __fmul_rn(xi, scale));
}

inline unsigned blocks(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

int cs_spec_windows(const uint8_t* plane, const uint32_t* vmask, int N, int overlap, int K, int nspec, int window,
                    const float lut[4], float* out, cudaStream_t st)
{
    if (!plane || !out || N % (16 * overlap) || (uintptr_t)plane % 4) return CS_ERR_ARG;
    const float* win = cs_window_table(window, N);
    if (!win) return CS_ERR_ARG;
    const int novl = overlap * K - (overlap - 1);
    const int64_t nwin = (int64_t)nspec * novl;
    k_spec_windows<<<blocks(nwin * (N / 16), 256), 256, 0, st>>>(reinterpret_cast<const uint32_t*>(plane), vmask, N,
                                                                 N / overlap, novl, (int64_t)K * N, nwin, win, lut[0],
                                                                 lut[1], lut[2], lut[3], out),
        cs_count_launches(1);
    return (int)cudaGetLastError();
}

int cs_xpol_reduce(const float2* X0, const float2* X1, int N, int overlap, int K, int nspec, float* power,
                   float2* xpol, cudaStream_t st)
{
    if (!X0 || !X1 || !power || !xpol) return CS_ERR_ARG;
    const int novl = overlap * K - (overlap - 1), nb = N / 2 + 1;
    const float scale = (float)(1.0 / (double)novl);
    const int64_t n = (int64_t)nspec * nb;
    k_xpol_reduce<<<blocks(n, 256), 256, 0, st>>>(X0, X1, nspec, novl, nb, scale, power, power + n, xpol),
        cs_count_launches(1);
    return (int)cudaGetLastError();
}
