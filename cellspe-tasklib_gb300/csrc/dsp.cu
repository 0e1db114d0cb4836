// Vector primitives behind the task-API commands of cellspe-tasklib-dsp.h.
//   MAC      acc += a*b            do_complex_mac  cellspe-tasklib-dsp.cpp:454-514
//   MAC conj acc += a*conj(b)      genericAddProduct_32fc_conj architecture.h:427-433
//   MULC     out = a*b             genericMul_32fc architecture.h:270-278
//   ADDC     out = a+b
//   SINCOS   {cos x, sin x}        exec_sincos :704-719, genericSinCos_32f :492-500
//   SINCOS_NORM  {cos 2 pi x, sin 2 pi x}   exec_sincosnormalized (:874-977)
//   SINCOS_GENERTR {cos, sin}(start + n*inc) exec_sincos_generator (:725-804)
//   autocorrelation accumulate acc.re += |x|^2  do_complex_autocorrelation (:431-449)
//   FADD     acc += x (floats)   ippsAdd_32f_I of TaskCoreIPP::combineResults
//                                 (spectrometer/src/IA-32/TaskCoreIPP.cpp:311-349)
// Each MAC/MUL keeps the reference's operand order and rounds every product
// and sum separately (__fmul_rn/__fadd_rn stop the compiler from fusing them
// into FMAs), so the FP32 results are bit-identical to the scalar generic
// loops of the reference.
#include "common.cuh"
#include "kernels.h"

namespace {
constexpr int NT = 256;

template <int OP>
__global__ void k_cvec(const float2* __restrict__ a, const float2* __restrict__ b, float2* __restrict__ o, int64_t n)
{
    int64_t i = (int64_t)blockIdx.x * NT + threadIdx.x;
    if (i >= n) return;
    float2 x = a[i], y = b[i];
    if constexpr (OP == 0) {          // acc += a*b
        float2 acc = o[i];
        acc.x = __fadd_rn(acc.x, __fsub_rn(__fmul_rn(x.x, y.x), __fmul_rn(x.y, y.y)));
        acc.y = __fadd_rn(acc.y, __fadd_rn(__fmul_rn(x.y, y.x), __fmul_rn(x.x, y.y)));
        o[i] = acc;
    } else if constexpr (OP == 1) {   // acc += a*conj(b)
        float2 acc = o[i];
        acc.x = __fadd_rn(acc.x, __fadd_rn(__fmul_rn(x.x, y.x), __fmul_rn(x.y, y.y)));
        acc.y = __fadd_rn(acc.y, __fsub_rn(__fmul_rn(x.y, y.x), __fmul_rn(x.x, y.y)));
        o[i] = acc;
    } else if constexpr (OP == 2) {   // out = a*b
        o[i] = make_float2(__fsub_rn(__fmul_rn(x.x, y.x), __fmul_rn(x.y, y.y)),
                           __fadd_rn(__fmul_rn(x.y, y.x), __fmul_rn(x.x, y.y)));
    } else {                          // out = a+b
        o[i] = make_float2(__fadd_rn(x.x, y.x), __fadd_rn(x.y, y.y));
    }
}

__global__ void k_sincos(const float* __restrict__ arg, float2* __restrict__ o, int64_t n, int normalized)
{
    int64_t i = (int64_t)blockIdx.x * NT + threadIdx.x;
    if (i >= n) return;
    float s, c;
    if (normalized) sincospif(2.0f * arg[i], &s, &c);
    else sincosf(arg[i], &s, &c);
    o[i] = make_float2(c, s);
}

__global__ void k_sincos_gen(double start, double inc, float2* __restrict__ o, int64_t n)
{
    int64_t i = (int64_t)blockIdx.x * NT + threadIdx.x;
    if (i >= n) return;
    double s, c;
    sincos(start + (double)i * inc, &s, &c);
    o[i] = make_float2((float)c, (float)s);
}

__global__ void k_autocorr(const float2* __restrict__ x, float2* __restrict__ acc, int64_t n)
{
    int64_t i = (int64_t)blockIdx.x * NT + threadIdx.x;
    if (i >= n) return;
    float2 v = x[i], a = acc[i];
    a.x = __fadd_rn(a.x, __fmul_rn(v.x, v.x));
    a.x = __fadd_rn(a.x, __fmul_rn(v.y, v.y));
    acc[i] = a;
}

__global__ void k_fadd(const float* __restrict__ x, float* __restrict__ acc, int64_t n)
{
    int64_t i = (int64_t)blockIdx.x * NT + threadIdx.x;
    if (i < n) acc[i] = __fadd_rn(acc[i], x[i]);
}

__global__ void k_recip(const float* __restrict__ in, float* __restrict__ out, int64_t n)
{
    int64_t i = (int64_t)blockIdx.x * NT + threadIdx.x;
    if (i < n) out[i] = 1.0f / in[i];
}

inline unsigned nblk(int64_t n) { return (unsigned)((n + NT - 1) / NT); }
}  // namespace

int cs_cmac(const float2* a, const float2* b, float2* acc, int64_t n, int conj_b, cudaStream_t st)
{
    if (n <= 0) return n == 0 ? 0 : CS_ERR_ARG;
    if (conj_b) k_cvec<1><<<nblk(n), NT, 0, st>>>(a, b, acc, n), cs_count_launches(1);
    else k_cvec<0><<<nblk(n), NT, 0, st>>>(a, b, acc, n), cs_count_launches(1);
    return (int)cudaGetLastError();
}

int cs_cmul(const float2* a, const float2* b, float2* out, int64_t n, cudaStream_t st)
{
    if (n <= 0) return n == 0 ? 0 : CS_ERR_ARG;
    k_cvec<2><<<nblk(n), NT, 0, st>>>(a, b, out, n), cs_count_launches(1);
    return (int)cudaGetLastError();
}

int cs_cadd(const float2* a, const float2* b, float2* out, int64_t n, cudaStream_t st)
{
    if (n <= 0) return n == 0 ? 0 : CS_ERR_ARG;
    k_cvec<3><<<nblk(n), NT, 0, st>>>(a, b, out, n), cs_count_launches(1);
    return (int)cudaGetLastError();
}

int cs_sincos(const float* arg, float2* cossin, int64_t n, int normalized, cudaStream_t st)
{
    if (n <= 0) return n == 0 ? 0 : CS_ERR_ARG;
    k_sincos<<<nblk(n), NT, 0, st>>>(arg, cossin, n, normalized), cs_count_launches(1);
    return (int)cudaGetLastError();
}

int cs_sincos_generator(float start, float inc, float2* cossin, int64_t n, cudaStream_t st)
{
    if (n <= 0) return n == 0 ? 0 : CS_ERR_ARG;
    k_sincos_gen<<<nblk(n), NT, 0, st>>>((double)start, (double)inc, cossin, n), cs_count_launches(1);
    return (int)cudaGetLastError();
}

int cs_autocorr_acc(const float2* x, float2* acc, int64_t n, cudaStream_t st)
{
    if (n <= 0) return n == 0 ? 0 : CS_ERR_ARG;
    k_autocorr<<<nblk(n), NT, 0, st>>>(x, acc, n), cs_count_launches(1);
    return (int)cudaGetLastError();
}

int cs_fadd(const float* x, float* acc, int64_t n, cudaStream_t st)
{
    if (n <= 0) return n == 0 ? 0 : CS_ERR_ARG;
    k_fadd<<<nblk(n), NT, 0, st>>>(x, acc, n), cs_count_launches(1);
    return (int)cudaGetLastError();
}

int cs_reciprocal(const float* in, float* out, int64_t n, cudaStream_t st)
{
    if (n <= 0) return n == 0 ? 0 : CS_ERR_ARG;
    k_recip<<<nblk(n), NT, 0, st>>>(in, out, n), cs_count_launches(1);
    return (int)cudaGetLastError();
}
