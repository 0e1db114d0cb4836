// K-a + K-b + K-c fused: the FX F stage.
//
// One CTA takes G consecutive segments of one input.  For each segment a
// group of M/16 threads (M = N/2) decodes the 2-bit samples straight into
// registers (LUT), runs the M-point complex FFT of z[n] = x[2n] + i x[2n+1]
// in shared memory, splits it into the N/2 channels of the real FFT (the
// Nyquist bin is dropped, as DiFX and zerocorr do), multiplies channel c by
// the delay/fringe phasor exp(i*(phase0 + c*dphase)) and an optional
// per-(input, channel) scale, and parks the result in a shared staging tile.
// The CTA then writes the tile out corner-turned (channel-major, time
// innermost) so that the X stage reads contiguous runs of time samples:
//   F32: float2 [C][S][K]        F16: __half [C][2][S][K] (re plane, im plane)
//
// Reference semantics: the per-segment order of exec_difxprocess
// (cellspe-tasklib-dsp.cpp:609-698) and do_runall_test (:1280-1308): integer
// (coarse) delay by shifting the read position, FFT, fractional-delay and
// fringe phasor multiply (complexfracmult, genericMul_32fc
// architecture.h:270-278).  The delay model itself is evaluated in FP64 by
// k_delay_state below.
#include "common.cuh"
#include "kernels.h"

namespace {

template <int M> struct FCfg {
    static constexpr int T = M / 16;
    static constexpr int GROUPS = (T >= 256) ? 1 : 256 / T;
    static constexpr int NT = T * GROUPS;
    static constexpr int RAWW = M / 8 + 2;     // 32-bit raw words staged per segment
};

template <int M, int FMT>
constexpr int stage_g()
{
    // segments per CTA: keeps the staging tile near 64 KB
    constexpr int elem = (FMT == CS_SPECTRA_F32) ? 8 : 4;
    constexpr int g = (64 * 1024) / (M * elem);
    return g >= 16 ? 16 : (g >= 8 ? 8 : (g >= 4 ? 4 : (g >= 2 ? 2 : 1)));
}

template <int M, int FMT>
size_t fstage_smem()
{
    using C = FCfg<M>;
    constexpr int G = stage_g<M, FMT>();
    size_t elem = (FMT == CS_SPECTRA_F32) ? 8 : 4;
    size_t stage = (G == 1) ? 0 : (size_t)M * (G + 1) * elem;   // G == 1: direct stores
    return (size_t)C::GROUPS * fpad_size(M) * 8 + (size_t)C::GROUPS * C::RAWW * 4 + stage;
}

CS_DEV float lut_pick(const float (&l)[4], unsigned c)
{
    float lo = (c & 1u) ? l[1] : l[0];
    float hi = (c & 1u) ? l[3] : l[2];
    return (c & 2u) ? hi : lo;
}

template <int M, int FMT, bool PHASE>
__global__ void __launch_bounds__(FCfg<M>::NT) k_fx_fstage(CsFStageArgs a, const float2* __restrict__ tw)
{
    using Cfg = FCfg<M>;
    constexpr int T = Cfg::T, GROUPS = Cfg::GROUPS, N = 2 * M;
    constexpr int G = stage_g<M, FMT>();
    extern __shared__ __align__(16) unsigned char smem[];
    float2* fbuf_all = reinterpret_cast<float2*>(smem);
    uint32_t* rbuf_all = reinterpret_cast<uint32_t*>(fbuf_all + GROUPS * fpad_size(M));
    unsigned char* stage = reinterpret_cast<unsigned char*>(rbuf_all + GROUPS * Cfg::RAWW);

    const int s = blockIdx.y;
    const int k0 = blockIdx.x * G;
    const int g = threadIdx.x / T, t = threadIdx.x % T;
    float2* fb = fbuf_all + g * fpad_size(M);
    uint32_t* rb = rbuf_all + g * Cfg::RAWW;
    auto bar = [&]() {
        if constexpr (GROUPS == 1) __syncthreads();
        else named_bar(1 + g, T);
    };
    const int64_t words = a.bytes_per_input >> 2;
    const uint32_t* src_in = reinterpret_cast<const uint32_t*>(a.raw + (int64_t)s * a.bytes_per_input);
    const bool msb = a.msb_first != 0;
    const float lut[4] = {a.lut[0], a.lut[1], a.lut[2], a.lut[3]};
    constexpr bool DIRECT = (G == 1);

    for (int ls = g; ls < G; ls += GROUPS) {
        const int k = k0 + ls;
        if (k >= a.K) break;                       // uniform over the group
        const int64_t sk = (int64_t)s * a.K + k;
        int64_t start = a.start_sample + (int64_t)k * N + (a.shift ? a.shift[sk] : 0);
        int64_t w0 = start >> 4;                   // floor for negative starts too
        int off = (int)(start & 15);
        for (int i = t; i < M / 8 + 1; i += T) {
            int64_t wi = w0 + i;
            rb[i] = (wi >= 0 && wi < words) ? __ldg(src_in + wi) : 0u;
        }
        bar();
        float2 v[16];
#pragma unroll
        for (int r = 0; r < 16; r++) {
            int n0 = off + 2 * (t + r * T);
            int n1 = n0 + 1;
            unsigned c0 = code2(rb[n0 >> 4], n0 & 15, msb);
            unsigned c1 = code2(rb[n1 >> 4], n1 & 15, msb);
            v[r] = make_float2(lut_pick(lut, c0), lut_pick(lut, c1));
        }
        CtaFft<M>::run(fb, t, v, tw, 2, bar);

        // phasor recurrences: channel kk = t + q*T and its mirror M - kk
        float2 A = make_float2(1.f, 0.f), B = A, D = A, AM = A;
        if constexpr (PHASE) {
            float ph0 = a.phase0[sk], dph = a.dphase[sk];
            float sn, cs;
            sincosf(ph0, &sn, &cs);             A = make_float2(cs, sn);
            sincosf((float)t * dph, &sn, &cs);  B = make_float2(cs, sn);
            sincosf((float)T * dph, &sn, &cs);  D = make_float2(cs, sn);
            sincosf((float)M * dph, &sn, &cs);  AM = cmul(A, make_float2(cs, sn));
        }
        const float* scl = a.scale ? a.scale + (int64_t)s * M : nullptr;
        auto emit = [&](int c, float2 X) {
            if (scl) X = cscale(X, __ldg(scl + c));
            if constexpr (DIRECT) {
                if constexpr (FMT == CS_SPECTRA_F32) {
                    reinterpret_cast<float2*>(a.out)[((int64_t)c * a.S + s) * a.K + k] = X;
                } else {
                    __half* o = reinterpret_cast<__half*>(a.out);
                    o[(((int64_t)c * 2 + 0) * a.S + s) * a.K + k] = __float2half_rn(X.x);
                    o[(((int64_t)c * 2 + 1) * a.S + s) * a.K + k] = __float2half_rn(X.y);
                }
            } else if constexpr (FMT == CS_SPECTRA_F32) {
                reinterpret_cast<float2*>(stage)[c * (G + 1) + ls] = X;
            } else {
                reinterpret_cast<__half2*>(stage)[c * (G + 1) + ls] = __floats2half2_rn(X.x, X.y);
            }
        };
#pragma unroll
        for (int q = 0; q <= (M / 2) / T; q++) {
            int kk = t + q * T;
            if (kk <= M / 2) {
                float2 Xk, Xm;
                r2c_pair(fb[fpad(kk)], fb[fpad((M - kk) & (M - 1))], twiddle(tw, kk), Xk, Xm);
                if constexpr (PHASE) {
                    Xk = cmul(Xk, cmul(A, B));
                    Xm = cmul(Xm, cmul_conj(AM, B));
                    B = cmul(B, D);
                }
                emit(kk, Xk);
                if (kk > 0 && kk < M / 2) emit(M - kk, Xm);
            }
        }
        bar();
    }
    if constexpr (DIRECT) return;
    __syncthreads();

    // ---- write the staging tile out, corner-turned ----
    const int nvalid = min(G, a.K - k0);
    const int S = a.S, K = a.K;
    if constexpr (FMT == CS_SPECTRA_F32) {
        const float2* st = reinterpret_cast<const float2*>(stage);
        float2* out = reinterpret_cast<float2*>(a.out);
        if (nvalid == G && (G % 2 == 0) && (K % 2 == 0)) {
            constexpr int P2 = G / 2;
            for (int idx = threadIdx.x; idx < M * P2; idx += Cfg::NT) {
                int c = idx / P2, l = 2 * (idx % P2);
                float2 x0 = st[c * (G + 1) + l], x1 = st[c * (G + 1) + l + 1];
                *reinterpret_cast<float4*>(out + ((int64_t)c * S + s) * K + k0 + l) =
                    make_float4(x0.x, x0.y, x1.x, x1.y);
            }
        } else {
            for (int idx = threadIdx.x; idx < M * G; idx += Cfg::NT) {
                int c = idx / G, l = idx % G;
                if (l < nvalid) out[((int64_t)c * S + s) * K + k0 + l] = st[c * (G + 1) + l];
            }
        }
    } else {
        const __half2* st = reinterpret_cast<const __half2*>(stage);
        __half* out = reinterpret_cast<__half*>(a.out);
        if (nvalid == G && (G % 8 == 0) && (K % 8 == 0)) {
            constexpr int P8 = G / 8;
            for (int idx = threadIdx.x; idx < M * 2 * P8; idx += Cfg::NT) {
                int l = 8 * (idx % P8);
                int plane = (idx / P8) & 1;
                int c = idx / (2 * P8);
                __align__(16) __half h[8];
#pragma unroll
                for (int j = 0; j < 8; j++) {
                    __half2 x = st[c * (G + 1) + l + j];
                    h[j] = plane ? __high2half(x) : __low2half(x);
                }
                *reinterpret_cast<uint4*>(out + (((int64_t)c * 2 + plane) * S + s) * K + k0 + l) =
                    *reinterpret_cast<const uint4*>(h);
            }
        } else {
            for (int idx = threadIdx.x; idx < M * 2 * G; idx += Cfg::NT) {
                int l = idx % G, plane = (idx / G) & 1, c = idx / (2 * G);
                if (l < nvalid) {
                    __half2 x = st[c * (G + 1) + l];
                    out[(((int64_t)c * 2 + plane) * S + s) * K + k0 + l] = plane ? __high2half(x) : __low2half(x);
                }
            }
        }
    }
}

template <int M, int FMT, bool PHASE>
int launch_fstage(const CsFStageArgs& a, cudaStream_t st)
{
    using Cfg = FCfg<M>;
    constexpr int G = stage_g<M, FMT>();
    const float2* tw = cs_twiddles(2 * M);
    if (!tw) return CS_ERR_ARG;
    size_t smem = fstage_smem<M, FMT>();
    auto kern = k_fx_fstage<M, FMT, PHASE>;
    CS_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    dim3 grid((a.K + G - 1) / G, a.S);
    kern<<<grid, Cfg::NT, smem, st>>>(a, tw), cs_count_launches(1);
    return (int)cudaGetLastError();
}

template <int M>
int dispatch_fstage(const CsFStageArgs& a, cudaStream_t st)
{
    bool ph = a.phase0 != nullptr;
    if (a.format == CS_SPECTRA_F32)
        return ph ? launch_fstage<M, CS_SPECTRA_F32, true>(a, st) : launch_fstage<M, CS_SPECTRA_F32, false>(a, st);
    return ph ? launch_fstage<M, CS_SPECTRA_F16, true>(a, st) : launch_fstage<M, CS_SPECTRA_F16, false>(a, st);
}

// ---------------------------------------------------------------------------
// N = 2048 fast path: one warp per segment.  The 1024-point complex FFT of
// z[n] = x[2n] + i x[2n+1] runs as a 32 x 32 four-step transform held in
// registers (each lane keeps 32 points): DFT-32 over n2 for n = lane + 32 n2,
// twiddle W_1024^(lane k1), one padded shared-memory transpose, DFT-32 over
// n1; lane l then holds Z[l + 32 k2].  The real-FFT split pairs Z[k] with
// Z[1024-k], which lives in lane (32-l) mod 32, register 31-k2 (lane 0:
// register (32-k2) mod 32), so it is a register shuffle.  Twiddles and
// delay phasors come from short register recurrences seeded from the FP64
// table.  Each CTA stages GW = 8 segments and writes them corner-turned.
// Input must be LSB-first (sample j of a 32-bit word at bits 2j).
// ---------------------------------------------------------------------------
constexpr int W_G = 8, W_WARPS = 8, W_TP = 33, W_RAWW = 2048 / 16 + 2;

template <int FMT>
size_t w2048_smem()
{
    size_t elem = (FMT == CS_SPECTRA_F32) ? 8 : 4;
    return (size_t)W_WARPS * 32 * W_TP * 8 + (size_t)W_WARPS * W_RAWW * 4 + (size_t)1024 * (W_G + 1) * elem;
}

template <int FMT, bool PHASE>
__global__ void __launch_bounds__(256, 2) k_fx_fstage_w2048(CsFStageArgs a, const float2* __restrict__ tw)
{
    constexpr int M = 1024, N = 2048, G = W_G;
    extern __shared__ __align__(16) unsigned char smem[];
    float2* tb_all = reinterpret_cast<float2*>(smem);
    uint32_t* rb_all = reinterpret_cast<uint32_t*>(tb_all + W_WARPS * 32 * W_TP);
    unsigned char* stage = reinterpret_cast<unsigned char*>(rb_all + W_WARPS * W_RAWW);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float2* tb = tb_all + warp * 32 * W_TP;
    uint32_t* rb = rb_all + warp * W_RAWW;
    const int s = blockIdx.y;
    const int k0 = blockIdx.x * G;
    const int k = k0 + warp;
    const float lut[4] = {a.lut[0], a.lut[1], a.lut[2], a.lut[3]};

    if (k < a.K) {
        const int64_t sk = (int64_t)s * a.K + k;
        const int64_t start = a.start_sample + (int64_t)k * N + (a.shift ? a.shift[sk] : 0);
        const int64_t w0 = start >> 4;
        const int off = (int)(start & 15);
        const int64_t words = a.bytes_per_input >> 2;
        const uint32_t* src = reinterpret_cast<const uint32_t*>(a.raw + (int64_t)s * a.bytes_per_input);
        for (int i = lane; i < W_RAWW; i += 32) {
            int64_t wi = w0 + i;
            rb[i] = (wi >= 0 && wi < words) ? __ldg(src + wi) : 0u;
        }
        __syncwarp();
        // decode: z[lane + 32 n2] uses samples off + 2 lane + 64 n2 (+1)
        const int f0 = off + 2 * lane;
        const int wb = f0 >> 4, sh = 2 * (f0 & 15);
        float2 v[32];
#pragma unroll
        for (int n2 = 0; n2 < 32; n2++) {
            uint32_t bits = __funnelshift_r(rb[wb + 4 * n2], rb[wb + 4 * n2 + 1], sh);
            v[n2] = make_float2(lut_pick(lut, bits & 3u), lut_pick(lut, (bits >> 2) & 3u));
        }
        // step 1: DFT-32 over n2 -> k1
        Dft<32>::run(v);
        // step 2: v[k1] *= W_1024^(lane k1) = (W_2048^(2 lane))^k1
        {
            const float2 w1 = twiddle(tw, 2 * lane);
            float2 wp[32];
            wp[1] = w1;
#pragma unroll
            for (int e = 2; e < 32; e++) wp[e] = (e & 1) ? cmul(wp[e - 1], w1) : cmul(wp[e / 2], wp[e / 2]);
#pragma unroll
            for (int e = 1; e < 32; e++) v[e] = cmul(v[e], wp[e]);
        }
        // transpose through shared memory: lane <- k1, register <- n1
#pragma unroll
        for (int e = 0; e < 32; e++) tb[e * W_TP + lane] = v[e];
        __syncwarp();
#pragma unroll
        for (int e = 0; e < 32; e++) v[e] = tb[lane * W_TP + e];
        // step 3: DFT-32 over n1 -> k2 ; v[k2] = Z[lane + 32 k2]
        Dft<32>::run(v);

        // real-FFT split, phasor, scale, stage
        const float2 wl = twiddle(tw, lane);                  // W_2048^lane
        float2 B = make_float2(1.f, 0.f), D = B;
        if constexpr (PHASE) {
            const float ph0 = a.phase0[sk], dph = a.dphase[sk];
            float sn, cs;
            sincosf(ph0 + (float)lane * dph, &sn, &cs);
            B = make_float2(cs, sn);
            sincosf(32.f * dph, &sn, &cs);
            D = make_float2(cs, sn);
        }
        const float* scl = a.scale ? a.scale + (int64_t)s * M : nullptr;
        const int src_lane = (32 - lane) & 31;
#pragma unroll
        for (int k2 = 0; k2 < 32; k2++) {
            float2 zb;
            zb.x = __shfl_sync(0xffffffffu, v[31 - k2].x, src_lane);
            zb.y = __shfl_sync(0xffffffffu, v[31 - k2].y, src_lane);
            if (lane == 0) zb = v[(32 - k2) & 31];
            const float2 za = v[k2];
            const float2 E = make_float2(0.5f * (za.x + zb.x), 0.5f * (za.y - zb.y));
            const float2 O = make_float2(0.5f * (za.y + zb.y), -0.5f * (za.x - zb.x));
            const float2 wk = cmul(wl, w64c(k2));          // W_2048^(lane + 32 k2)
            float2 X = cadd(E, cmul(wk, O));
            const int c = lane + 32 * k2;
            if constexpr (PHASE) {
                X = cmul(X, B);
                B = cmul(B, D);
            }
            if (scl) X = cscale(X, __ldg(scl + c));
            if constexpr (FMT == CS_SPECTRA_F32)
                reinterpret_cast<float2*>(stage)[c * (G + 1) + warp] = X;
            else
                reinterpret_cast<__half2*>(stage)[c * (G + 1) + warp] = __floats2half2_rn(X.x, X.y);
        }
    }
    __syncthreads();

    // corner-turned write-out
    const int nvalid = min(G, a.K - k0);
    const int S = a.S, K = a.K;
    if constexpr (FMT == CS_SPECTRA_F32) {
        const float2* st = reinterpret_cast<const float2*>(stage);
        float2* out = reinterpret_cast<float2*>(a.out);
        if (nvalid == G && K % 2 == 0) {
            for (int idx = threadIdx.x; idx < M * (G / 2); idx += 256) {
                int c = idx / (G / 2), l = 2 * (idx % (G / 2));
                float2 x0 = st[c * (G + 1) + l], x1 = st[c * (G + 1) + l + 1];
                *reinterpret_cast<float4*>(out + ((int64_t)c * S + s) * K + k0 + l) = make_float4(x0.x, x0.y, x1.x, x1.y);
            }
        } else {
            for (int idx = threadIdx.x; idx < M * G; idx += 256) {
                int c = idx / G, l = idx % G;
                if (l < nvalid) out[((int64_t)c * S + s) * K + k0 + l] = st[c * (G + 1) + l];
            }
        }
    } else {
        const __half2* st = reinterpret_cast<const __half2*>(stage);
        __half* out = reinterpret_cast<__half*>(a.out);
        if (nvalid == G && K % 8 == 0) {
            for (int idx = threadIdx.x; idx < M * 2; idx += 256) {
                int plane = idx & 1, c = idx >> 1;
                __align__(16) __half h[8];
#pragma unroll
                for (int j = 0; j < 8; j++) {
                    __half2 x = st[c * (G + 1) + j];
                    h[j] = plane ? __high2half(x) : __low2half(x);
                }
                *reinterpret_cast<uint4*>(out + (((int64_t)c * 2 + plane) * S + s) * K + k0) =
                    *reinterpret_cast<const uint4*>(h);
            }
        } else {
            for (int idx = threadIdx.x; idx < M * 2 * G; idx += 256) {
                int l = idx % G, plane = (idx / G) & 1, c = idx / (2 * G);
                if (l < nvalid) {
                    __half2 x = st[c * (G + 1) + l];
                    out[(((int64_t)c * 2 + plane) * S + s) * K + k0 + l] = plane ? __high2half(x) : __low2half(x);
                }
            }
        }
    }
}

template <int FMT, bool PHASE>
int launch_w2048(const CsFStageArgs& a, cudaStream_t st)
{
    const float2* tw = cs_twiddles(2048);
    if (!tw) return CS_ERR_ARG;
    size_t smem = w2048_smem<FMT>();
    auto kern = k_fx_fstage_w2048<FMT, PHASE>;
    CS_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    dim3 grid((a.K + W_G - 1) / W_G, a.S);
    kern<<<grid, 256, smem, st>>>(a, tw), cs_count_launches(1);
    return (int)cudaGetLastError();
}

// FP64 delay model (kept in FP64 on the GPU: the fringe phase 2 pi f_LO tau
// spans ~1e7 cycles for millisecond delays at GHz sky frequencies, far beyond
// FP32's 24-bit mantissa).  Operations are written out with explicit
// rounding so the result matches a plain FP64 evaluation on the host.
__global__ void k_delay_state(const double* __restrict__ poly, int S, int N, int K, double fs, double lo,
                              CsDelayState ds)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)S * K) return;
    int s = (int)(i / K), k = (int)(i % K);
    double t = __ddiv_rn(__dadd_rn(__dmul_rn((double)k, (double)N), (double)N / 2.0), fs);
    const double* c = poly + 4 * s;
    double tau = 0.0;
    for (int m = 3; m >= 0; m--) tau = __dadd_rn(__dmul_rn(tau, t), c[m]);
    double sh = rint(__dmul_rn(tau, fs));
    double frac = __dsub_rn(tau, __ddiv_rn(sh, fs));
    double cyc = __dmul_rn(lo, tau);
    const double twopi = 6.283185307179586;
    double ph0 = __dmul_rn(twopi, __dsub_rn(cyc, floor(cyc)));
    double dph = __dmul_rn(__dmul_rn(twopi, __ddiv_rn(fs, (double)N)), frac);
    ds.shift[i] = (int32_t)sh;
    ds.phase0[i] = (float)ph0;
    ds.dphase[i] = (float)dph;
}

}  // namespace

int cs_delay_state(const double* poly, int S, int N, int K, double fs_hz, double lo_hz, CsDelayState ds,
                   cudaStream_t st)
{
    int64_t n = (int64_t)S * K;
    if (n <= 0) return CS_ERR_ARG;
    k_delay_state<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(poly, S, N, K, fs_hz, lo_hz, ds), cs_count_launches(1);
    return (int)cudaGetLastError();
}

int cs_fx_fstage(const CsFStageArgs& a, cudaStream_t st)
{
    if (!a.raw || !a.out || a.S <= 0 || a.K <= 0) return CS_ERR_ARG;
    if ((uintptr_t)a.raw % 16 || a.bytes_per_input % 16 || (uintptr_t)a.out % 16) return CS_ERR_ARG;
    if (a.N == 2048 && !a.msb_first) {
        const bool ph = a.phase0 != nullptr;
        if (a.format == CS_SPECTRA_F32)
            return ph ? launch_w2048<CS_SPECTRA_F32, true>(a, st) : launch_w2048<CS_SPECTRA_F32, false>(a, st);
        return ph ? launch_w2048<CS_SPECTRA_F16, true>(a, st) : launch_w2048<CS_SPECTRA_F16, false>(a, st);
    }
    switch (a.N) {
        case 1024: return dispatch_fstage<512>(a, st);
        case 2048: return dispatch_fstage<1024>(a, st);
        case 4096: return dispatch_fstage<2048>(a, st);
        case 8192: return dispatch_fstage<4096>(a, st);
        case 16384: return dispatch_fstage<8192>(a, st);
        case 32768: return dispatch_fstage<16384>(a, st);
        default: return CS_ERR_UNSUPPORTED;
    }
}
