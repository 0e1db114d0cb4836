// Shared device helpers for the GB300 FX correlator / spectrometer kernels.
//
// * complex float helpers (float2: x = re, y = im)
// * radix-2/4/8/16 DFT codelets held in registers (forward, e^{-2 pi i nk/R},
//   unscaled -- the convention of fft_1d_r2_modified.h:40-66 and exec_FFT,
//   cellspe-tasklib-dsp.cpp:519-584)
// * CtaFft<M>: an M-point complex Stockham autosort FFT run by M/16 threads
//   that each hold 16 points; passes exchange through padded shared memory.
#pragma once
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <stdint.h>

#define CS_DEV __device__ __forceinline__

// Window weight of sample i of an n-point FFT for the spectrometer's window
// types, which are the reference's WindowFunctionType (spectrometer
// Settings.h: 0 None, 1 Cosine, 2 Cosine2, 3 Hamming, 4 Hann, 5 Blackman), in
// FP64 (callers round to FP32).  Cosine and Cosine2 are
// TaskCoreIPP::generate_windowfunction's own loops (TaskCoreIPP.cpp:569-605,
// i and n rounded to FP32 in the argument); Hamming, Hann and Blackman are the
// IPP windows it calls (ippsWinHamming_32f_I, ippsWinHann_32f_I,
// ippsWinBlackman_32f_I with alpha 0.5), from IPP's published definitions
// with x = 2 pi i / (n - 1): 0.54 - 0.46 cos x; 0.5 - 0.5 cos x;
// (alpha + 1)/2 - 0.5 cos x - (alpha/2) cos 2x.  Any other type is 1.0.
__host__ __device__ inline double cs_window_value(int type, int i, int n)
{
    if (type == 1 || type == 2) {
        const double arg = 3.14159265358979323846 * ((double)(float)i - 0.5 * (double)(float)n + 0.5) / (double)(float)n;
        const double c = cos(arg);
        return type == 1 ? (double)(float)c : c * c;
    }
    const double x = 2.0 * 3.14159265358979323846 * (double)i / (double)(n - 1);
    if (type == 3) return 0.54 - 0.46 * cos(x);
    if (type == 4) return 0.5 - 0.5 * cos(x);
    if (type == 5) return 0.75 - 0.5 * cos(x) - 0.25 * cos(2.0 * x);
    return 1.0;
}

CS_DEV float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
CS_DEV float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
CS_DEV float2 cmul(float2 a, float2 b)
{
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
CS_DEV float2 cmul_conj(float2 a, float2 b)  // a * conj(b)
{
    return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
CS_DEV float2 mul_mi(float2 a) { return make_float2(a.y, -a.x); }   // a * (-i)
CS_DEV float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }

// cos(r pi / 16), r = 0..8 and cos(r pi / 32), r = 0..16 (constant bank:
// indices are warp-uniform, so reads broadcast).
static __constant__ float c_cos32[9] = {1.0f, 0.98078528040323043f, 0.92387953251128674f, 0.83146961230254524f, 0.70710678118654757f, 0.55557023301960229f, 0.38268343236508984f, 0.19509032201612833f, 0.0f};
static __constant__ float c_cos64[17] = {1.0f, 0.99518472667219693f, 0.98078528040323043f, 0.95694033573220882f, 0.92387953251128674f, 0.88192126434835505f, 0.83146961230254524f, 0.77301045336273699f, 0.70710678118654757f, 0.63439328416364549f, 0.55557023301960229f, 0.47139673682599781f, 0.38268343236508984f, 0.29028467725446233f, 0.19509032201612833f, 0.09801714032956077f, 0.0f};

// W32^m = exp(-2 pi i m / 32), m in [0, 32).
CS_DEV float2 w32(int m)
{
    m &= 31;
    const int q = m >> 3, r = m & 7;          // quadrant, offset inside it
    const float cr = c_cos32[r], sr = c_cos32[8 - r];
    // exp(-i (q*pi/2 + r*pi/16)) = (-i)^q * (cr - i sr)
    float2 z = make_float2(cr, -sr);
    switch (q) {
        case 0: return z;
        case 1: return make_float2(z.y, -z.x);
        case 2: return make_float2(-z.x, -z.y);
        default: return make_float2(-z.y, z.x);
    }
}
CS_DEV float2 w16(int m) { return w32(2 * m); }

// W64^m = exp(-2 pi i m / 64) for m in [0, 32).
CS_DEV float2 w64c(int m)
{
    const int q = (m >> 4) & 1, r = m & 15;
    float2 z = make_float2(c_cos64[r], -c_cos64[16 - r]);
    return q ? make_float2(z.y, -z.x) : z;
}

// v * W32^e with the exact quarter turns kept exact (e folds to a constant
// inside unrolled codelets, so the switch disappears).
CS_DEV float2 rot32(float2 v, int e)
{
    switch (e & 31) {
        case 0: return v;
        case 8: return make_float2(v.y, -v.x);
        case 16: return make_float2(-v.x, -v.y);
        case 24: return make_float2(-v.y, v.x);
        default: return cmul(v, w32(e));
    }
}

CS_DEV void dft2(float2& a, float2& b)
{
    float2 t = a;
    a = cadd(t, b);
    b = csub(t, b);
}

// In-place forward DFT of R points in natural order.
template <int R> struct Dft;

template <> struct Dft<1> {
    static CS_DEV void run(float2*) {}
};
template <> struct Dft<2> {
    static CS_DEV void run(float2* a) { dft2(a[0], a[1]); }
};
template <> struct Dft<4> {
    static CS_DEV void run(float2* a)
    {
        float2 t0 = cadd(a[0], a[2]), t1 = csub(a[0], a[2]);
        float2 t2 = cadd(a[1], a[3]), t3 = mul_mi(csub(a[1], a[3]));
        a[0] = cadd(t0, t2);
        a[2] = csub(t0, t2);
        a[1] = cadd(t1, t3);
        a[3] = csub(t1, t3);
    }
};
// R = R1*R2 split: n = R2*n1 + n2, k = k1 + R1*k2.
template <int R1, int R2> struct DftSplit {
    static CS_DEV void run(float2* a)
    {
        constexpr int R = R1 * R2;
        float2 b[R2][R1];
#pragma unroll
        for (int n2 = 0; n2 < R2; n2++) {
#pragma unroll
            for (int n1 = 0; n1 < R1; n1++) b[n2][n1] = a[R2 * n1 + n2];
            Dft<R1>::run(b[n2]);
#pragma unroll
            for (int k1 = 0; k1 < R1; k1++) b[n2][k1] = rot32(b[n2][k1], (n2 * k1) * (32 / R));
        }
#pragma unroll
        for (int k1 = 0; k1 < R1; k1++) {
            float2 c[R2];
#pragma unroll
            for (int n2 = 0; n2 < R2; n2++) c[n2] = b[n2][k1];
            Dft<R2>::run(c);
#pragma unroll
            for (int k2 = 0; k2 < R2; k2++) a[k1 + R1 * k2] = c[k2];
        }
    }
};
template <> struct Dft<8> {
    static CS_DEV void run(float2* a) { DftSplit<2, 4>::run(a); }
};
template <> struct Dft<16> {
    static CS_DEV void run(float2* a) { DftSplit<4, 4>::run(a); }
};
template <> struct Dft<32> {
    static CS_DEV void run(float2* a) { DftSplit<4, 8>::run(a); }
};

// Padded shared-memory index: one spare float2 after every 16 elements keeps
// the stride-16 accesses of the radix-16 passes free of bank conflicts.
CS_DEV int fpad(int i) { return i + (i >> 4); }
__host__ __device__ constexpr int fpad_size(int m) { return m + m / 16; }

// exp(-2 pi i m / L) from a table of L entries computed in FP64 on the host.
CS_DEV float2 twiddle(const float2* __restrict__ tw, int m) { return __ldg(tw + m); }

// ---------------------------------------------------------------------------
// CtaFft<M>: M-point complex forward FFT by a group of T = M/16 threads.
//   Stage 0 (first pass, NS = 1) starts from registers: thread t holds
//   v[r] = z[t + r*T], r = 0..15.  Each later pass reads 16 points per thread
//   from the padded buffer, applies twiddles W_{NS*R}^{r*k}, runs a radix-R
//   codelet and writes back (Stockham autosort: the result ends up in natural
//   order).  The caller provides the group-wide barrier.
// ---------------------------------------------------------------------------
// TWREC: each butterfly loads one twiddle w from the table and forms w^2..w^15
// by a balanced recurrence (w^2e = (w^e)^2, w^(2e+1) = w^2e w: at most four
// products deep), trading table loads for FMA work.  Used for transforms of
// 2048 points and more, whose tables no longer stay in L1.
template <int M, bool TWREC = false> struct CtaFft {
    static_assert(M >= 16 && (M & (M - 1)) == 0, "M must be a power of two >= 16");
    static constexpr int T = M / 16;

    // First pass: radix-16 butterflies on register data, output to buf.
    static CS_DEV void first_pass(float2* buf, int t, float2 (&v)[16])
    {
        Dft<16>::run(v);
#pragma unroll
        for (int r = 0; r < 16; r++) buf[fpad(16 * t + r)] = v[r];
    }

    // One Stockham pass with stride NS (> 1) and radix R = min(16, M/NS).
    // tw is exp(-2 pi i m / (M*tws)) for m in [0, M*tws): the table of a
    // larger transform is shared by striding it.
    template <int NS, class Barrier>
    static CS_DEV void pass(float2* buf, int t, const float2* __restrict__ tw, int tws, Barrier bar)
    {
        constexpr int R = (M / NS >= 16) ? 16 : (M / NS);
        constexpr int NB = M / R;          // butterflies in this pass
        constexpr int PER = NB / T;        // butterflies per thread = 16 / R
        float2 v[PER][R];
#pragma unroll
        for (int q = 0; q < PER; q++) {
            int j = t + q * T;
#pragma unroll
            for (int r = 0; r < R; r++) v[q][r] = buf[fpad(j + r * NB)];
        }
        bar();
#pragma unroll
        for (int q = 0; q < PER; q++) {
            int j = t + q * T;
            int k = j & (NS - 1);
            constexpr int STEP = M / (NS * R);
            if constexpr (TWREC) {
                float2 wp[R];
                wp[1] = twiddle(tw, k * STEP * tws);
#pragma unroll
                for (int e = 2; e < R; e++) wp[e] = (e & 1) ? cmul(wp[e - 1], wp[1]) : cmul(wp[e / 2], wp[e / 2]);
#pragma unroll
                for (int r = 1; r < R; r++) v[q][r] = cmul(v[q][r], wp[r]);
            } else {
#pragma unroll
                for (int r = 1; r < R; r++) v[q][r] = cmul(v[q][r], twiddle(tw, (r * k) * STEP * tws));
            }
            Dft<R>::run(v[q]);
            int base = (j - k) * R + k;
#pragma unroll
            for (int r = 0; r < R; r++) buf[fpad(base + r * NS)] = v[q][r];
        }
        bar();
    }

    template <int NS, class Barrier>
    static CS_DEV void rest(float2* buf, int t, const float2* __restrict__ tw, int tws, Barrier bar)
    {
        if constexpr (NS < M) {
            pass<NS>(buf, t, tw, tws, bar);
            constexpr int R = (M / NS >= 16) ? 16 : (M / NS);
            rest<NS * R>(buf, t, tw, tws, bar);
        }
    }

    // Full transform: v holds z[t + r*T]; on return buf holds Z (natural
    // order, padded indexing) and every thread has passed the final barrier.
    template <class Barrier>
    static CS_DEV void run(float2* buf, int t, float2 (&v)[16], const float2* __restrict__ tw,
                           int tws, Barrier bar)
    {
        first_pass(buf, t, v);
        bar();
        rest<16>(buf, t, tw, tws, bar);
    }
};

// Named barrier over `nthreads` threads (a multiple of 32) with id `id`.
CS_DEV void named_bar(int id, int nthreads)
{
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

// 2-bit field extraction.  Sample j (0..15) of a little-endian 32-bit word:
// LSB-first order keeps it at bits 2j; MSB-first order (sample 0 in bits 7:6
// of each byte) keeps it at bits 8*(j/4) + 6 - 2*(j%4).
CS_DEV unsigned code2(uint32_t w, int j, bool msb_first)
{
    int sh = msb_first ? (8 * (j >> 2) + 6 - 2 * (j & 3)) : (2 * j);
    return (w >> sh) & 3u;
}

// Error-check helper for host code in .cu files.
#define CS_CUDA_TRY(expr)                                   \
    do {                                                    \
        cudaError_t _e = (expr);                            \
        if (_e != cudaSuccess) return (int)_e;              \
    } while (0)

// Real-to-complex split.  Z is the M-point FFT of z[n] = x[2n] + i x[2n+1]
// (N = 2M real points).  With a = Z[k], b = Z[(M-k) mod M] and
// w = exp(-2 pi i k / N):  E = (a + conj b)/2,  O = (a - conj b)/(2i),
//   X[k] = E + w O,   X[M-k] = conj(E - w O).
CS_DEV void r2c_pair(float2 a, float2 b, float2 w, float2& Xk, float2& Xmk)
{
    float2 E = make_float2(0.5f * (a.x + b.x), 0.5f * (a.y - b.y));
    float2 O = make_float2(0.5f * (a.y + b.y), -0.5f * (a.x - b.x));
    float2 wO = cmul(w, O);
    Xk = cadd(E, wO);
    float2 d = csub(E, wO);
    Xmk = make_float2(d.x, -d.y);
}
