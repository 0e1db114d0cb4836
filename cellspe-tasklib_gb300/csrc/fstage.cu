// K-a + K-b + K-c fused: the FX F stage.
//
// Every kernel here decodes the 2-bit samples, transforms each segment (the
// N-point real FFT as an M = N/2-point complex FFT of z[n] = x[2n] + i x[2n+1]
// and a split), applies the channel phasor and scale, and writes FP32 or FP16
// spectra for the X stage.  Which kernel runs (cs_fx_fstage):
//   N = 512      k_fx_fstage_w512    a half-warp per segment, 16 points per lane
//   N = 1024     k_fx_fstage_w1024   a half-warp per segment, 32 points per lane
//   N = 2048     k_fx_fstage_w2048   a warp per segment (five CTA schedules, timed)
//   N >= 4096    k_fx_fstage_wbig    N/2048 warps per segment, segment-major out
//                                    (cs_spectra_transpose makes the X-stage rows)
//   MSB-first input, or CELLSPE_FSTAGE_GENERIC=1: k_fx_fstage, described next.
//
// k_fx_fstage: one CTA takes G consecutive segments of one input.  For each segment a
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

#include <algorithm>
#include <cstdlib>
#include <mutex>

namespace {

CS_DEV int out_pitch(const CsFStageArgs& a) { return a.kp ? a.kp : a.K; }
CS_DEV int out_rows(const CsFStageArgs& a) { return a.S_out ? a.S_out : a.S; }

template <int M> struct FCfg {
    static constexpr int T = M / 16;
    static constexpr int GROUPS = (T >= 256) ? 1 : 256 / T;
    static constexpr int NT = T * GROUPS;
    static constexpr int RAWW = M / 8 + 2;     // 32-bit raw words staged per segment
    // groups narrower than a warp cannot use named barriers: the whole CTA
    // then advances in lockstep on __syncthreads
    static constexpr bool CTA_BAR = (GROUPS == 1) || (T < 32);
};

template <int M, int FMT>
constexpr int stage_g()
{
    // segments per CTA: keeps the staging tile near 64 KB
    constexpr int elem = (FMT == CS_SPECTRA_F32) ? 8 : 4;
    constexpr int g = (64 * 1024) / (M * elem);
    return g >= 16 ? 16 : (g >= 8 ? 8 : (g >= 4 ? 4 : (g >= 2 ? 2 : 1)));
}

template <int M, int FMT, bool SEGMAJ>
size_t fstage_smem()
{
    using C = FCfg<M>;
    constexpr int G = SEGMAJ ? 1 : stage_g<M, FMT>();
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

template <int M, int FMT, bool PHASE, bool SEGMAJ>
__global__ void __launch_bounds__(FCfg<M>::NT) k_fx_fstage(const __grid_constant__ CsFStageArgs a, const float2* __restrict__ tw)
{
    using Cfg = FCfg<M>;
    constexpr int T = Cfg::T, GROUPS = Cfg::GROUPS, N = 2 * M;
    constexpr int G = SEGMAJ ? 1 : stage_g<M, FMT>();
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
        if constexpr (Cfg::CTA_BAR) __syncthreads();
        else named_bar(1 + g, T);
    };
    const int64_t words = a.bytes_per_input >> 2;
    const uint32_t* src_in = reinterpret_cast<const uint32_t*>(a.raw + (int64_t)s * a.bytes_per_input);
    const bool msb = a.msb_first != 0;
    const float lut[4] = {a.lut[0], a.lut[1], a.lut[2], a.lut[3]};
    constexpr bool DIRECT = (G == 1);
    // LSB-first input: a sample pair's 4 bits index a table of level pairs
    __shared__ float2 lut16[16];
    if (threadIdx.x < 16) lut16[threadIdx.x] = make_float2(lut[threadIdx.x & 3], lut[threadIdx.x >> 2]);
    __syncthreads();

    // every group runs the same number of rounds (barriers stay uniform);
    // segments past K are computed on zeros and not stored
    for (int ls = g; ls < ((G + GROUPS - 1) / GROUPS) * GROUPS; ls += GROUPS) {
        const int k = k0 + ls;
        const bool valid = (ls < G) && (k < a.K);
        const int64_t sk = (int64_t)s * a.K + (valid ? k : 0);
        int64_t start = a.start_sample + (int64_t)(valid ? k : 0) * N + (a.shift ? a.shift[sk] : 0);
        int64_t w0 = start >> 4;                   // floor for negative starts too
        int off = (int)(start & 15);
        for (int i = t; i < Cfg::RAWW; i += T) {
            int64_t wi = w0 + i;
            rb[i] = (valid && wi >= 0 && wi < words) ? __ldg(src_in + wi) : 0u;
        }
        bar();
        float2 v[16];
        if (!msb) {
#pragma unroll
            for (int r = 0; r < 16; r++) {
                const int n0 = off + 2 * (t + r * T);         // the pair may straddle two words
                v[r] = lut16[__funnelshift_r(rb[n0 >> 4], rb[(n0 >> 4) + 1], 2 * (n0 & 15)) & 15u];
            }
        } else {
#pragma unroll
            for (int r = 0; r < 16; r++) {
                int n0 = off + 2 * (t + r * T);
                int n1 = n0 + 1;
                unsigned c0 = code2(rb[n0 >> 4], n0 & 15, msb);
                unsigned c1 = code2(rb[n1 >> 4], n1 & 15, msb);
                v[r] = make_float2(lut_pick(lut, c0), lut_pick(lut, c1));
            }
        }
        CtaFft<M, (M >= 2048)>::run(fb, t, v, tw, 2, bar);

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
            if (!valid) return;
            if (scl) X = cscale(X, __ldg(scl + c));
            if constexpr (SEGMAJ) {
                const int64_t i = ((int64_t)s * a.K + k) * M + c;      // [S][K][C], coalesced in c
                if constexpr (FMT == CS_SPECTRA_F32) reinterpret_cast<float2*>(a.out)[i] = X;
                else reinterpret_cast<__half2*>(a.out)[i] = __floats2half2_rn(X.x, X.y);
            } else if constexpr (DIRECT) {
                if constexpr (FMT == CS_SPECTRA_F32) {
                    reinterpret_cast<float2*>(a.out)[((int64_t)c * out_rows(a) + s) * out_pitch(a) + k] = X;
                } else {
                    __half* o = reinterpret_cast<__half*>(a.out);
                    o[(((int64_t)c * 2 + 0) * out_rows(a) + s) * out_pitch(a) + k] = __float2half_rn(X.x);
                    o[(((int64_t)c * 2 + 1) * out_rows(a) + s) * out_pitch(a) + k] = __float2half_rn(X.y);
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
    const int S = out_rows(a), KP = out_pitch(a);      // output layout
    if constexpr (FMT == CS_SPECTRA_F32) {
        const float2* st = reinterpret_cast<const float2*>(stage);
        float2* out = reinterpret_cast<float2*>(a.out);
        if (nvalid == G && (G % 2 == 0) && (KP % 2 == 0)) {
            constexpr int P2 = G / 2;
            for (int idx = threadIdx.x; idx < M * P2; idx += Cfg::NT) {
                int c = idx / P2, l = 2 * (idx % P2);
                float2 x0 = st[c * (G + 1) + l], x1 = st[c * (G + 1) + l + 1];
                *reinterpret_cast<float4*>(out + ((int64_t)c * S + s) * KP + k0 + l) =
                    make_float4(x0.x, x0.y, x1.x, x1.y);
            }
        } else {
            for (int idx = threadIdx.x; idx < M * G; idx += Cfg::NT) {
                int c = idx / G, l = idx % G;
                if (l < nvalid) out[((int64_t)c * S + s) * KP + k0 + l] = st[c * (G + 1) + l];
            }
        }
    } else {
        const __half2* st = reinterpret_cast<const __half2*>(stage);
        __half* out = reinterpret_cast<__half*>(a.out);
        if (nvalid == G && (G % 8 == 0) && (KP % 8 == 0)) {
            constexpr int P8 = G / 8;
            for (int idx = threadIdx.x; idx < M * 2 * P8; idx += Cfg::NT) {
                int l = 8 * (idx % P8);
                int plane = (idx / P8) & 1;
                int c = idx / (2 * P8);
                // pick the Re (low) or Im (high) halves of 8 staged half2 words
                const uint32_t* w = reinterpret_cast<const uint32_t*>(st + c * (G + 1) + l);
                const uint32_t sel = plane ? 0x7632u : 0x5410u;
                *reinterpret_cast<uint4*>(out + (((int64_t)c * 2 + plane) * S + s) * KP + k0 + l) =
                    make_uint4(__byte_perm(w[0], w[1], sel), __byte_perm(w[2], w[3], sel),
                               __byte_perm(w[4], w[5], sel), __byte_perm(w[6], w[7], sel));
            }
        } else {
            for (int idx = threadIdx.x; idx < M * 2 * G; idx += Cfg::NT) {
                int l = idx % G, plane = (idx / G) & 1, c = idx / (2 * G);
                if (l < nvalid) {
                    __half2 x = st[c * (G + 1) + l];
                    out[(((int64_t)c * 2 + plane) * S + s) * KP + k0 + l] = plane ? __high2half(x) : __low2half(x);
                }
            }
        }
    }
}

template <int M, int FMT, bool PHASE, bool SEGMAJ>
int launch_fstage(const CsFStageArgs& a, cudaStream_t st)
{
    using Cfg = FCfg<M>;
    constexpr int G = SEGMAJ ? 1 : stage_g<M, FMT>();
    const float2* tw = cs_twiddles(2 * M);
    if (!tw) return CS_ERR_ARG;
    size_t smem = fstage_smem<M, FMT, SEGMAJ>();
    auto kern = k_fx_fstage<M, FMT, PHASE, SEGMAJ>;
    CS_CUDA_TRY(cs_smem_at_least(reinterpret_cast<const void*>(kern), (int)smem));
    dim3 grid((a.K + G - 1) / G, a.S);
    kern<<<grid, Cfg::NT, smem, st>>>(a, tw), cs_count_launches(1);
    return (int)cudaGetLastError();
}

template <int M, bool SEGMAJ>
int dispatch_fstage2(const CsFStageArgs& a, cudaStream_t st)
{
    bool ph = a.phase0 != nullptr;
    if (a.format == CS_SPECTRA_F32)
        return ph ? launch_fstage<M, CS_SPECTRA_F32, true, SEGMAJ>(a, st)
                  : launch_fstage<M, CS_SPECTRA_F32, false, SEGMAJ>(a, st);
    return ph ? launch_fstage<M, CS_SPECTRA_F16, true, SEGMAJ>(a, st)
              : launch_fstage<M, CS_SPECTRA_F16, false, SEGMAJ>(a, st);
}

// Segment-major output only from 2048-point complex transforms (N >= 4096):
// the staged corner turn there holds at most 4 segments (8-byte runs).
template <int M>
int dispatch_fstage(const CsFStageArgs& a, cudaStream_t st)
{
    if constexpr (M >= 2048) {
        if (a.seg_major) return dispatch_fstage2<M, true>(a, st);
    } else {
        if (a.seg_major) return CS_ERR_ARG;
    }
    return dispatch_fstage2<M, false>(a, st);
}

// ---------------------------------------------------------------------------
// N = 2048 fast path: one warp per segment.
// The 1024-point complex FFT of z[n] = x[2n] + i x[2n+1] runs as a 32 x 32
// four-step transform held in registers (each lane keeps 32 points): DFT-32
// over n2 for n = lane + 32 n2, twiddle W_1024^(lane k1) from a shared table,
// one padded shared-memory transpose (one float plane at a time), DFT-32 over
// n1; lane l then holds Z[l + 32 k2].  The real-FFT split pairs Z[k] with
// Z[1024-k], which lives in lane (32-l) mod 32, register 31-k2 (lane 0:
// register (32-k2) mod 32), so it is a register shuffle.  A CTA of WARPS
// warps stages W_G = 8 segments of one input and writes them corner-turned;
// with WARPS = 4 each warp transforms two segments and fetches the raw words
// of the second with cp.async while it transforms the first.
// Input must be LSB-first (sample j of a 32-bit word at bits 2j).
// ---------------------------------------------------------------------------
constexpr int W_G = 8, W_TP = 33;
constexpr int W_RAWC = 2048 / 64 + 2;          // 16-byte chunks staged per segment (34 = 136 words)
constexpr int W_RAWW = 4 * W_RAWC;

template <int FMT, int WARPS, int G>
size_t w2048_smem()
{
    size_t elem = (FMT == CS_SPECTRA_F32) ? 8 : 4;
    return (size_t)WARPS * 32 * W_TP * 8            // transpose tiles (complex)
           + (size_t)WARPS * 2 * W_RAWW * 4         // raw double buffers
           + 16 * 8                                 // pair LUT
           + (size_t)1024 * (G + 1) * elem;         // staging tile
}

CS_DEV void cp_async16(uint32_t dst, const void* src, bool valid)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(valid ? 16 : 0)
                 : "memory");
}
CS_DEV void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N_PENDING>
CS_DEV void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N_PENDING) : "memory"); }

template <int FMT, bool PHASE, int WARPS, int ROUNDS, int G>
__global__ void __launch_bounds__(32 * WARPS, (WARPS == 16 || G > 16) ? 1 : (WARPS == 8) ? 2 : 3) k_fx_fstage_w2048(const __grid_constant__ CsFStageArgs a, const float2* __restrict__ tw)
{
    constexpr int M = 1024, N = 2048, NT = 32 * WARPS, PER = G / WARPS;
    static_assert(G % WARPS == 0 && G % 8 == 0, "segments per CTA");
    extern __shared__ __align__(16) unsigned char smem[];
    float2* tb_all = reinterpret_cast<float2*>(smem);
    uint32_t* rb_all = reinterpret_cast<uint32_t*>(tb_all + WARPS * 32 * W_TP);
    float2* lut16 = reinterpret_cast<float2*>(rb_all + WARPS * 2 * W_RAWW);
    unsigned char* stage = reinterpret_cast<unsigned char*>(lut16 + 16);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float2* tb = tb_all + warp * 32 * W_TP;
    uint32_t* rb = rb_all + warp * 2 * W_RAWW;
    const int s = blockIdx.y;
    const int kbase = blockIdx.x * G * ROUNDS;
    const int64_t chunks = a.bytes_per_input >> 4;
    const unsigned char* base = a.raw + (int64_t)s * a.bytes_per_input;

    // raw words of this warp's u-th segment (round u / PER, slot u % PER) ->
    // buffer u & 1 (cp.async, zero fill outside the input); returns the sample
    // offset inside the staged words
    auto prefetch = [&](int u) -> int {
        const int r = u % PER, round = u / PER;
        const int k = kbase + round * G + warp + WARPS * r;
        const bool kv = k < a.K;
        const int64_t start = a.start_sample + (int64_t)k * N + ((a.shift && kv) ? __ldg(a.shift + (int64_t)s * a.K + k) : 0);
        const int64_t c0 = start >> 6;
        const uint32_t dst = (uint32_t)__cvta_generic_to_shared(rb + (u & 1) * W_RAWW);
        for (int c = lane; c < W_RAWC; c += 32) {
            const int64_t ci = c0 + c;
            const bool ok = kv && ci >= 0 && ci < chunks;
            cp_async16(dst + 16 * c, ok ? base + 16 * ci : a.raw, ok);
        }
        cp_async_commit();
        return (int)(start & 63);
    };
    int off_next = prefetch(0);

    // per-lane twiddle seeds, computed in place (no global loads while the
    // raw words arrive): W_1024^lane for the four-step twiddles, W_2048^lane / 2
    // for the real-FFT split
    if (threadIdx.x < 16) lut16[threadIdx.x] = make_float2(a.lut[threadIdx.x & 3], a.lut[threadIdx.x >> 2]);
    float2 w1, whalf;
    {
        float sn, cs;
        sincospif(-(float)lane / 512.0f, &sn, &cs);
        w1 = make_float2(cs, sn);
        sincospif(-(float)lane / 1024.0f, &sn, &cs);
        whalf = make_float2(0.5f * cs, 0.5f * sn);
    }
    // W_1024^(lane e), e < 16, by a balanced recurrence (w^2e = (w^e)^2,
    // w^(2e+1) = w^2e w), and W_1024^(16 lane), kept for all segments
    float2 wp[16];
    wp[0] = make_float2(1.f, 0.f);
    wp[1] = w1;
#pragma unroll
    for (int e = 2; e < 16; e++) wp[e] = (e & 1) ? cmul(wp[e - 1], w1) : cmul(wp[e / 2], wp[e / 2]);
    const float2 w16p = cmul(wp[8], wp[8]);
    __syncthreads();
    const int src_lane = (32 - lane) & 31;

#pragma unroll 1
    for (int round = 0; round < ROUNDS; round++) {
    const int k0 = kbase + round * G;
#pragma unroll 1
    for (int r = 0; r < PER; r++) {
        const int u = round * PER + r;
        const int ls = warp + WARPS * r;
        const int k = k0 + ls;
        const int off = off_next;
        if (u + 1 < PER * ROUNDS) {
            off_next = prefetch(u + 1);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncwarp();
        if (k < a.K) {
            const int64_t sk = (int64_t)s * a.K + k;
            const uint32_t* rw = rb + (u & 1) * W_RAWW;
            const int f0 = off + 2 * lane;
            const int wb = f0 >> 4, sh = 2 * (f0 & 15);
            float2 v[32];
#pragma unroll
            for (int n2 = 0; n2 < 32; n2++) {
                const uint32_t bits = __funnelshift_r(rw[wb + 4 * n2], rw[wb + 4 * n2 + 1], sh);
                v[n2] = lut16[bits & 15u];
            }
            Dft<32>::run(v);                                    // over n2 -> k1
            // v[k1] *= W_1024^(lane k1), the powers formed once per thread
#pragma unroll
            for (int e = 1; e < 16; e++) v[e] = cmul(v[e], wp[e]);
            v[16] = cmul(v[16], w16p);
#pragma unroll
            for (int e = 17; e < 32; e++) v[e] = cmul(v[e], cmul(w16p, wp[e - 16]));
#pragma unroll
            for (int e = 0; e < 32; e++) tb[e * W_TP + lane] = v[e];
            __syncwarp();
#pragma unroll
            for (int e = 0; e < 32; e++) v[e] = tb[lane * W_TP + e];
            __syncwarp();
            Dft<32>::run(v);                                    // over n1 -> k2: v[k2] = Z[lane + 32 k2]

            // Real-FFT split, one pair (k, 1024 - k) per lane and step: with
            // s = Z[k] + conj(Z[1024-k]), d = Z[k] - conj(Z[1024-k]) and
            // t = (W_2048^k / 2) d,
            //     X[k] = s/2 - i t,     X[1024-k] = conj(s/2 + i t)
            // (W_2048^(1024-k) = -conj(W_2048^k)).  Lane l, step k2 < 16 takes
            // k = l + 32 k2, whose partner Z[1024-k] is lane (32-l) mod 32's
            // register 31-k2 (lane 0: its own register (32-k2) mod 32); lane 0
            // adds the self-paired k = 512.  X[1024] (k = 0's partner) is not a
            // channel.  Optional per-channel phasor exp(i (ph0 + c dph)) and
            // scale, then the staging store.
            float2 B = make_float2(1.f, 0.f), D = B, B2 = B;
            if constexpr (PHASE) {
                const float ph0 = __ldg(a.phase0 + sk), dph = __ldg(a.dphase + sk);
                float sn, cs;
                sincosf(ph0 + (float)lane * dph, &sn, &cs);
                B = make_float2(cs, sn);                         // channel lane + 32 k2
                sincosf(ph0 + (float)(M - lane) * dph, &sn, &cs);
                B2 = make_float2(cs, sn);                        // channel 1024 - lane - 32 k2
                sincosf(32.f * dph, &sn, &cs);
                D = make_float2(cs, sn);
            }
            const float* scl = a.scale ? a.scale + (int64_t)s * M : nullptr;
            auto put = [&](int c, float2 X) {
                if (scl) X = cscale(X, __ldg(scl + c));
                if constexpr (FMT == CS_SPECTRA_F32)
                    reinterpret_cast<float2*>(stage)[c * (G + 1) + ls] = X;
                else
                    reinterpret_cast<__half2*>(stage)[c * (G + 1) + ls] = __floats2half2_rn(X.x, X.y);
            };
#pragma unroll
            for (int k2 = 0; k2 <= 16; k2++) {
                if (k2 == 16 && lane != 0) break;
                float2 zb;
                if (k2 < 16) {
                    zb.x = __shfl_sync(0xffffffffu, v[31 - k2].x, src_lane);
                    zb.y = __shfl_sync(0xffffffffu, v[31 - k2].y, src_lane);
                }
                if (lane == 0) zb = v[(32 - k2) & 31];
                const float2 za = v[k2];
                const float2 sm = make_float2(za.x + zb.x, za.y - zb.y);
                const float2 df = make_float2(za.x - zb.x, za.y + zb.y);
                const float2 t = cmul(cmul(whalf, w64c(k2)), df);
                float2 X1 = make_float2(fmaf(0.5f, sm.x, t.y), fmaf(0.5f, sm.y, -t.x));
                float2 X2 = make_float2(fmaf(0.5f, sm.x, -t.y), -fmaf(0.5f, sm.y, t.x));
                const int c1 = lane + 32 * k2, c2 = M - c1;
                if constexpr (PHASE) {
                    X1 = cmul(X1, B);
                    X2 = cmul(X2, B2);
                    B = cmul(B, D);
                    B2 = cmul_conj(B2, D);
                }
                put(c1, X1);
                if (k2 < 16 && c1 != 0) put(c2, X2);
            }
        }
    }
    __syncthreads();

    // corner-turned write-out of the G staged segments
    const int nvalid = max(0, min(G, a.K - k0));
    const int S = out_rows(a), KP = out_pitch(a);      // output layout
    if constexpr (FMT == CS_SPECTRA_F32) {
        const float2* st = reinterpret_cast<const float2*>(stage);
        float2* out = reinterpret_cast<float2*>(a.out);
        if (nvalid == G && KP % 2 == 0) {
            for (int idx = threadIdx.x; idx < M * (G / 2); idx += NT) {
                const int c = idx / (G / 2), l = 2 * (idx % (G / 2));
                const float2 x0 = st[c * (G + 1) + l], x1 = st[c * (G + 1) + l + 1];
                *reinterpret_cast<float4*>(out + ((int64_t)c * S + s) * KP + k0 + l) = make_float4(x0.x, x0.y, x1.x, x1.y);
            }
        } else {
            for (int idx = threadIdx.x; idx < M * G; idx += NT) {
                const int c = idx / G, l = idx % G;
                if (l < nvalid) out[((int64_t)c * S + s) * KP + k0 + l] = st[c * (G + 1) + l];
            }
        }
    } else {
        const __half2* st = reinterpret_cast<const __half2*>(stage);
        __half* out = reinterpret_cast<__half*>(a.out);
        // element (c, plane, s, k): channel-major planes [C][2][S][KP], or
        // k-blocked [C][S][KP/32][2][32] (the Re and Im halves of 32 segments
        // side by side: a 32-segment tile writes 128 contiguous bytes per channel)
        auto at = [&](int c, int plane, int k) -> int64_t {
            if (a.kblock) return ((((int64_t)c * S + s) * (KP / 32) + k / 32) * 2 + plane) * 32 + (k % 32);
            return (((int64_t)c * 2 + plane) * S + s) * KP + k;
        };
        if (nvalid == G && KP % 8 == 0) {
            constexpr int P8 = G / 8;                 // 16-byte pieces per output row
            for (int idx = threadIdx.x; idx < M * 2 * P8; idx += NT) {
                const int piece = idx % P8, plane = (idx / P8) & 1, c = idx / (2 * P8);
                // pick the Re (low) or Im (high) halves of 8 staged half2 words
                const uint32_t* w = reinterpret_cast<const uint32_t*>(st + c * (G + 1) + 8 * piece);
                const uint32_t sel = plane ? 0x7632u : 0x5410u;
                *reinterpret_cast<uint4*>(out + at(c, plane, k0 + 8 * piece)) =
                    make_uint4(__byte_perm(w[0], w[1], sel), __byte_perm(w[2], w[3], sel),
                               __byte_perm(w[4], w[5], sel), __byte_perm(w[6], w[7], sel));
            }
        } else {
            for (int idx = threadIdx.x; idx < M * 2 * G; idx += NT) {
                const int l = idx % G, plane = (idx / G) & 1, c = idx / (2 * G);
                if (l < nvalid) {
                    const __half2 x = st[c * (G + 1) + l];
                    out[at(c, plane, k0 + l)] = plane ? __high2half(x) : __low2half(x);
                }
            }
        }
    }
    if (round + 1 < ROUNDS) __syncthreads();     // the staging tile is reused
    }
}

template <int FMT, bool PHASE, int WARPS, int ROUNDS, int G = W_G>
int launch_w2048_variant(const CsFStageArgs& a, const float2* tw, cudaStream_t st)
{
    size_t smem = w2048_smem<FMT, WARPS, G>();
    auto kern = k_fx_fstage_w2048<FMT, PHASE, WARPS, ROUNDS, G>;
    CS_CUDA_TRY(cs_smem_at_least(reinterpret_cast<const void*>(kern), (int)smem));
    dim3 grid((a.K + G * ROUNDS - 1) / (G * ROUNDS), a.S);
    kern<<<grid, 32 * WARPS, smem, st>>>(a, tw), cs_count_launches(1);
    return (int)cudaGetLastError();
}

constexpr int W_NVARIANTS = 5;

template <int FMT, bool PHASE>
int launch_w2048_choice(int choice, const CsFStageArgs& a, const float2* tw, cudaStream_t st)
{
    switch (choice) {
        case 2: return launch_w2048_variant<FMT, PHASE, 4, 1>(a, tw, st);
        case 3: return launch_w2048_variant<FMT, PHASE, 8, 2>(a, tw, st);
        case 4:
            // 16 warps, 16 segments: 32-byte output runs (FP16 staging fits)
            if constexpr (FMT == CS_SPECTRA_F16) return launch_w2048_variant<FMT, PHASE, 16, 1, 16>(a, tw, st);
            return launch_w2048_variant<FMT, PHASE, 8, 1>(a, tw, st);
        case 5:
            // 8 warps, 32 segments (4 per warp): 64-byte output runs
            if constexpr (FMT == CS_SPECTRA_F16) return launch_w2048_variant<FMT, PHASE, 8, 1, 32>(a, tw, st);
            return launch_w2048_variant<FMT, PHASE, 8, 1>(a, tw, st);
        default: return launch_w2048_variant<FMT, PHASE, 8, 1>(a, tw, st);
    }
}

// Schedule choice per (format, phase): 1 = 8 warps, one segment each;
// 2 = 4 warps, two segments each with the second prefetched; 3 = 8 warps,
// two rounds of 8 segments per CTA (the second round's raw words prefetched
// during the first); 4 = 16 warps and 16 segments per CTA, so that each
// output row gets a 32-byte run; 5 = 8 warps, 32 segments per CTA (64-byte
// runs, 128 in the k-blocked layout); 4 and 5 are FP16 only.
// The choice is timed on the caller's own job: every schedule computes the
// same values, so each is launched on the job's arguments (one warm-up and
// one timed launch) and the fastest kept (schedule 5 unless another is more
// than 2 % faster); the job's own launch follows.  Small jobs do not rank the
// schedules the way large ones do (on 128 inputs x 1024 segments schedules 2
// and 5 are within 2 %, on 512 x 4096 they are 5 % apart), so jobs under
// 2^16 input-segments never time, and a job with more than four times the
// segments of the one that was timed times them again.  The timing runs
// outside the lock: other threads keep launching the current choice
// meanwhile.  Never while the stream is being captured (the timing
// synchronises), nor on threads that turned timing off (the correlation
// service's workers: timing would add ten F-stage launches to a live job's
// latency); the environment variable CELLSPE_FSTAGE_VARIANT forces one.
struct W2048Choice {
    int variant = 0;
    int64_t work = 0;            // input-segments of the job it was timed on
    bool timing = false;         // a thread is timing the schedules now
};
W2048Choice g_w2048_choice[2][2];
std::mutex g_w2048_mu;
thread_local bool t_w2048_timing_allowed = true;
constexpr int64_t W_TUNE_MIN_WORK = 1 << 16;

template <int FMT, bool PHASE>
int tune_w2048(const CsFStageArgs& a, const float2* tw, cudaStream_t st)
{
    const int dflt = FMT == CS_SPECTRA_F16 ? 5 : 1;
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess) return dflt;
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return dflt;
    }
    float best = 1e30f;
    int choice = dflt;
    for (int v = 1; v <= W_NVARIANTS; v++) {
        if (FMT == CS_SPECTRA_F32 && v >= 4) break;        // 4 and 5 fall back to 1 for FP32
        float ms = 1e30f;
        if (launch_w2048_choice<FMT, PHASE>(v, a, tw, st) == 0) {
            cudaEventRecord(e0, st);
            const int rc = launch_w2048_choice<FMT, PHASE>(v, a, tw, st);
            cudaEventRecord(e1, st);
            if (cudaEventSynchronize(e1) == cudaSuccess && rc == 0) cudaEventElapsedTime(&ms, e0, e1);
        }
        cudaGetLastError();
        if (v == dflt) ms *= 0.98f;
        if (ms < best) { best = ms; choice = v; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return choice;
}

template <int FMT, bool PHASE>
int launch_w2048(const CsFStageArgs& a, cudaStream_t st)
{
    const float2* tw = cs_twiddles(2048);
    if (!tw) return CS_ERR_ARG;
    const char* env = getenv("CELLSPE_FSTAGE_VARIANT");
    if (env && env[0] >= '1' && env[0] <= '0' + W_NVARIANTS)
        return launch_w2048_choice<FMT, PHASE>(env[0] - '0', a, tw, st);
    W2048Choice& c = g_w2048_choice[FMT == CS_SPECTRA_F16][PHASE ? 1 : 0];
    const int64_t work = (int64_t)a.S * a.K;
    int variant;
    bool time_now = false;
    {
        std::lock_guard<std::mutex> lk(g_w2048_mu);
        variant = c.variant ? c.variant : (FMT == CS_SPECTRA_F16 ? 5 : 1);
        if (t_w2048_timing_allowed && !c.timing && work >= W_TUNE_MIN_WORK && (!c.variant || work > 4 * c.work)) {
            cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
            if (cudaStreamIsCapturing(st, &cap) == cudaSuccess && cap == cudaStreamCaptureStatusNone)
                time_now = c.timing = true;
            else
                cudaGetLastError();
        }
    }
    if (time_now) {
        variant = tune_w2048<FMT, PHASE>(a, tw, st);
        std::lock_guard<std::mutex> lk(g_w2048_mu);
        c.variant = variant;
        c.work = work;
        c.timing = false;
    }
    return launch_w2048_choice<FMT, PHASE>(variant, a, tw, st);
}


// ---------------------------------------------------------------------------
// N = 4096 ... 32768: M1 = M / 1024 warps per segment (M = N/2 complex points).
// Decimation in time by M1: warp n1 transforms x_n1[m] = z[n1 + M1 m],
// m < 1024, exactly as the 2048-point path does (lane l holds m = l + 32 j,
// DFT-32 over j, twiddle W_1024^(l k1), padded per-warp transpose, DFT-32), so
// lane l ends with Y_n1[l + 32 k2] in register k2.  The warps park Y_n1 in
// shared memory (the warp's own transpose tile) and, after one CTA barrier,
//     Z[k2 + 1024 k1] = sum_n1 W_M1^(n1 k1) (W_M^(n1 k2) Y_n1[k2]).
// Each thread takes the mirrored columns k2 and 1024 - k2 (k2 = 1 ... 511;
// thread 0 also columns 0 and 512): twiddled by powers of u = W_M^k2 (the
// second column by conj(u)^n1, whose DFT comes out rotated by one since
// W_M^(n1 (1024 - k2)) = W_M1^n1 conj(u)^n1), two M1-point DFTs, and the
// real-FFT split pairs Z[k2 + 1024 k1] with Z[M - k2 - 1024 k1] =
// Z[(1024 - k2) + 1024 (M1 - 1 - k1)], so the split needs no data exchange.
// Channels then get the phasor exp(i (phase0 + c dphase)) and the optional
// scale and are written segment-major ([S][K][C], coalesced along c) for
// cs_spectra_transpose.  LSB-first input only.  A CTA that fills an SM on its
// own (16 warps, or 8 warps with the phasor's registers) takes SEGS = 4
// consecutive segments and fetches the next one's raw words (cp.async) while
// it transforms the current one; the other forms take one segment and leave
// the overlap to the other CTAs on the SM.
// ---------------------------------------------------------------------------
constexpr int B_TILE = 32 * W_TP;               // float2 per warp: transpose tile, then Y_n1

template <int M1, bool PHASE>
constexpr int wbig_segs()
{
    return (M1 == 16 || (M1 == 8 && PHASE)) ? 4 : 1;
}

template <int M1, bool PHASE>
size_t wbig_smem()
{
    constexpr int bufs = wbig_segs<M1, PHASE>() > 1 ? 2 : 1;
    return (size_t)M1 * B_TILE * 8 + (size_t)bufs * (2048 * M1 / 64 + 2) * 16 + 16 * 8;
}

template <int M1, int FMT, bool PHASE>
__global__ void __launch_bounds__(32 * M1) k_fx_fstage_wbig(const __grid_constant__ CsFStageArgs a, const float2* __restrict__ tw)
{
    constexpr int M = 1024 * M1, N = 2 * M, NT = 32 * M1;
    constexpr int RAWC = N / 64 + 2;             // 16-byte chunks of one segment (+ alignment slack)
    constexpr int SEGS = wbig_segs<M1, PHASE>(), BUFS = SEGS > 1 ? 2 : 1;
    extern __shared__ __align__(16) unsigned char smem[];
    float2* tiles = reinterpret_cast<float2*>(smem);
    uint32_t* rw_all = reinterpret_cast<uint32_t*>(tiles + M1 * B_TILE);
    float2* lut16 = reinterpret_cast<float2*>(rw_all + BUFS * 4 * RAWC);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int s = blockIdx.y, kbase = blockIdx.x * SEGS;
    const int64_t chunks = a.bytes_per_input >> 4;
    const unsigned char* base = a.raw + (int64_t)s * a.bytes_per_input;

    // raw words of segment kbase + i -> buffer i % BUFS (zero fill outside the
    // input); returns the sample offset inside the staged words
    auto prefetch = [&](int i) -> int {
        const int k = kbase + i;
        const int64_t start = a.start_sample + (int64_t)k * N + (a.shift ? __ldg(a.shift + (int64_t)s * a.K + k) : 0);
        const int64_t c0 = start >> 6;
        const uint32_t dst = (uint32_t)__cvta_generic_to_shared(rw_all + (i % BUFS) * 4 * RAWC);
        for (int c = threadIdx.x; c < RAWC; c += NT) {
            const int64_t ci = c0 + c;
            const bool ok = ci >= 0 && ci < chunks;
            cp_async16(dst + 16 * c, ok ? base + 16 * ci : a.raw, ok);
        }
        cp_async_commit();
        return (int)(start & 63);
    };
    int off_next = prefetch(0);
    if (threadIdx.x < 16) lut16[threadIdx.x] = make_float2(a.lut[threadIdx.x & 3], a.lut[threadIdx.x >> 2]);
    // W_1024^(lane e): e < 8 by a balanced recurrence, then blocks of 8 by powers of W_1024^(8 lane)
    float2 wp[8];
    {
        float sn, cs;
        sincospif(-(float)lane / 512.0f, &sn, &cs);
        wp[0] = make_float2(1.f, 0.f);
        wp[1] = make_float2(cs, sn);
#pragma unroll
        for (int e = 2; e < 8; e++) wp[e] = (e & 1) ? cmul(wp[e - 1], wp[1]) : cmul(wp[e / 2], wp[e / 2]);
    }
    const float2 w8 = cmul(wp[4], wp[4]);
    float2* tb = tiles + warp * B_TILE;
    const float2 c2 = __ldg(tw + 1024);                          // W_N^1024 = W_(2 M1)

#pragma unroll 1
    for (int i = 0; i < SEGS; i++) {
    const int k = kbase + i;
    if (k >= a.K) break;                                         // uniform over the CTA
    const int64_t sk = (int64_t)s * a.K + k;
    const int off = off_next;
    if (i + 1 < SEGS && k + 1 < a.K) {
        off_next = prefetch(i + 1);
        cp_async_wait<1>();
    } else {
        cp_async_wait<0>();
    }
    __syncthreads();                 // raw words in; the previous segment's columns are read
    const uint32_t* rw = rw_all + (i % BUFS) * 4 * RAWC;

    // ---- warp n1: 1024-point transform of z[n1 + M1 m] ----
    {
        const int f0 = off + 2 * (warp + M1 * lane);            // sample offset of this lane's first pair
        const int wb = f0 >> 4, sh = 2 * (f0 & 15);
        float2 v[32];
#pragma unroll
        for (int j = 0; j < 32; j++) {                           // pair j is 64 M1 samples = 4 M1 words further on
            const uint32_t bits = __funnelshift_r(rw[wb + 4 * M1 * j], rw[wb + 4 * M1 * j + 1], sh);
            v[j] = lut16[bits & 15u];
        }
        Dft<32>::run(v);
        float2 q = make_float2(1.f, 0.f);
#pragma unroll
        for (int b = 0; b < 4; b++) {
#pragma unroll
            for (int r = 0; r < 8; r++) {
                if (b == 0 && r == 0) continue;
                v[8 * b + r] = cmul(v[8 * b + r], b ? cmul(q, wp[r]) : wp[r]);
            }
            q = b ? cmul(q, w8) : w8;
        }
#pragma unroll
        for (int e = 0; e < 32; e++) tb[e * W_TP + lane] = v[e];
        __syncwarp();
#pragma unroll
        for (int e = 0; e < 32; e++) v[e] = tb[lane * W_TP + e];
        __syncwarp();
        Dft<32>::run(v);                                         // v[k2] = Y_n1[lane + 32 k2]
#pragma unroll
        for (int e = 0; e < 32; e++) tb[lane + 32 * e] = v[e];
    }
    __syncthreads();

    // ---- mirrored column pairs: radix-M1 step, real-FFT split, phasor, write ----
    float2 D = make_float2(1.f, 0.f);
    float ph0 = 0.f, dph = 0.f;
    if constexpr (PHASE) {
        ph0 = __ldg(a.phase0 + sk);
        dph = __ldg(a.dphase + sk);
        float sn, cs;
        sincosf(1024.f * dph, &sn, &cs);
        D = make_float2(cs, sn);
    }
    const float* scl = a.scale ? a.scale + (int64_t)s * M : nullptr;
    const int64_t obase = sk * M;
    auto emit = [&](int c, float2 X) {
        if (scl) X = cscale(X, __ldg(scl + c));
        if constexpr (FMT == CS_SPECTRA_F32) reinterpret_cast<float2*>(a.out)[obase + c] = X;
        else reinterpret_cast<__half2*>(a.out)[obase + c] = __floats2half2_rn(X.x, X.y);
    };
    auto phasor = [&](int c) -> float2 {
        float sn, cs;
        sincosf(ph0 + (float)c * dph, &sn, &cs);
        return make_float2(cs, sn);
    };
#pragma unroll 1
    for (int task = threadIdx.x; task < 512; task += NT) {
        if (task == 0) {
            // column 0 (u = 1) and column 512 (u = W_M^512), each paired with itself
            float2 y0[M1], y5[M1];
            const float2 u = __ldg(tw + 1024);
            float2 p = make_float2(1.f, 0.f);
#pragma unroll
            for (int n1 = 0; n1 < M1; n1++) {
                y0[n1] = tiles[n1 * B_TILE];
                y5[n1] = cmul(tiles[n1 * B_TILE + 512], p);
                p = cmul(p, u);
            }
            Dft<M1>::run(y0);
            Dft<M1>::run(y5);
            float2 w = make_float2(1.f, 0.f);                    // W_N^(1024 k1)
#pragma unroll
            for (int k1 = 0; k1 <= M1 / 2; k1++) {
                float2 Xk, Xm;
                r2c_pair(y0[k1], y0[(M1 - k1) % M1], w, Xk, Xm);
                const int c = 1024 * k1;
                if constexpr (PHASE) Xk = cmul(Xk, phasor(c)), Xm = cmul(Xm, phasor(M - c));
                emit(c, Xk);
                if (k1 > 0 && k1 < M1 / 2) emit(M - c, Xm);
                w = cmul(w, c2);
            }
            w = __ldg(tw + 512);                                  // W_N^(512 + 1024 k1)
#pragma unroll
            for (int k1 = 0; k1 < M1 / 2; k1++) {
                float2 Xk, Xm;
                r2c_pair(y5[k1], y5[M1 - 1 - k1], w, Xk, Xm);
                const int c = 512 + 1024 * k1;
                if constexpr (PHASE) Xk = cmul(Xk, phasor(c)), Xm = cmul(Xm, phasor(M - c));
                emit(c, Xk);
                emit(M - c, Xm);
                w = cmul(w, c2);
            }
            continue;
        }
        const int kA = task, kB = 1024 - task;
        float2 ya[M1], yb[M1];
        {
            const float2 u = __ldg(tw + 2 * kA);                 // W_M^kA
            float2 p = make_float2(1.f, 0.f);
#pragma unroll
            for (int n1 = 0; n1 < M1; n1++) {
                ya[n1] = cmul(tiles[n1 * B_TILE + kA], p);
                yb[n1] = cmul_conj(tiles[n1 * B_TILE + kB], p);
                p = cmul(p, u);
            }
        }
        Dft<M1>::run(ya);                                         // ya[k1] = Z[kA + 1024 k1]
        Dft<M1>::run(yb);                                         // yb[(k1 + 1) % M1] = Z[kB + 1024 k1]
        float2 w = __ldg(tw + kA);                                // W_N^(kA + 1024 k1)
        float2 BA = make_float2(1.f, 0.f), BB = BA;
        if constexpr (PHASE) {
            BA = phasor(kA);                                      // channel kA + 1024 k1
            BB = phasor(M - kA);                                  // channel M - kA - 1024 k1
        }
#pragma unroll
        for (int k1 = 0; k1 < M1; k1++) {
            float2 Xk, Xm;
            r2c_pair(ya[k1], yb[(M1 - k1) % M1], w, Xk, Xm);
            const int c = kA + 1024 * k1;
            if constexpr (PHASE) {
                Xk = cmul(Xk, BA);
                Xm = cmul(Xm, BB);
                BA = cmul(BA, D);
                BB = cmul_conj(BB, D);
            }
            emit(c, Xk);
            emit(M - c, Xm);
            w = cmul(w, c2);
        }
    }
    }
}

template <int M1, int FMT, bool PHASE>
int launch_wbig(const CsFStageArgs& a, cudaStream_t st)
{
    const float2* tw = cs_twiddles(2048 * M1);
    if (!tw) return CS_ERR_ARG;
    constexpr int SEGS = wbig_segs<M1, PHASE>();
    const size_t smem = wbig_smem<M1, PHASE>();
    auto kern = k_fx_fstage_wbig<M1, FMT, PHASE>;
    CS_CUDA_TRY(cs_smem_at_least(reinterpret_cast<const void*>(kern), (int)smem));
    kern<<<dim3((a.K + SEGS - 1) / SEGS, a.S), 32 * M1, smem, st>>>(a, tw), cs_count_launches(1);
    return (int)cudaGetLastError();
}

template <int M1>
int dispatch_wbig(const CsFStageArgs& a, cudaStream_t st)
{
    const bool ph = a.phase0 != nullptr;
    if (a.format == CS_SPECTRA_F32)
        return ph ? launch_wbig<M1, CS_SPECTRA_F32, true>(a, st) : launch_wbig<M1, CS_SPECTRA_F32, false>(a, st);
    return ph ? launch_wbig<M1, CS_SPECTRA_F16, true>(a, st) : launch_wbig<M1, CS_SPECTRA_F16, false>(a, st);
}


// ---------------------------------------------------------------------------
// N = 512: one half-warp per segment.  The 256-point complex FFT of
// z[n] = x[2n] + i x[2n+1] runs as a 16 x 16 four-step held in registers:
// lane l of the half-warp keeps n = l + 16 j (j < 16), DFT-16 over j, twiddle
// W_256^(l k1), a padded 16 x 17 transpose, DFT-16, after which lane l holds
// Z[l + 16 k2].  The real-FFT split pairs Z[k] with Z[256 - k], which lives in
// lane (16 - l) mod 16 of the same half-warp, register 15 - k2 (lane 0: its
// own register (16 - k2) mod 16): a 16-wide shuffle.  A CTA of 8 warps
// stages 64 segments of one input (each half-warp four, the next one's raw
// words fetched with cp.async during the current transform) and writes them
// corner-turned: 128-byte runs per (channel, plane) row in FP16, 512 in FP32.
// The two half-warps of a warp fill staging columns 16 apart, so their
// stores fall in disjoint banks.  LSB-first input only.
// ---------------------------------------------------------------------------
// Corner-turned write-out of a staging tile [M channels][G + 1] (G segments of
// input s from segment k0; FP32 float2 or FP16 half2 Re|Im) into the channel-
// major layout: F32 float2 rows (c, s), F16 half rows (c, plane, s), pitch KP.
template <int FMT, int M, int G, int NT>
CS_DEV void stage_writeout(const CsFStageArgs& a, const unsigned char* stage, int s, int k0)
{
    const int nvalid = max(0, min(G, a.K - k0));
    const int S = out_rows(a), KP = out_pitch(a);
    if constexpr (FMT == CS_SPECTRA_F32) {
        const float2* st = reinterpret_cast<const float2*>(stage);
        float2* out = reinterpret_cast<float2*>(a.out);
        if (nvalid == G && KP % 2 == 0) {
            for (int idx = threadIdx.x; idx < M * (G / 2); idx += NT) {
                const int c = idx / (G / 2), l = 2 * (idx % (G / 2));
                const float2 x0 = st[c * (G + 1) + l], x1 = st[c * (G + 1) + l + 1];
                *reinterpret_cast<float4*>(out + ((int64_t)c * S + s) * KP + k0 + l) = make_float4(x0.x, x0.y, x1.x, x1.y);
            }
        } else {
            for (int idx = threadIdx.x; idx < M * G; idx += NT) {
                const int c = idx / G, l = idx % G;
                if (l < nvalid) out[((int64_t)c * S + s) * KP + k0 + l] = st[c * (G + 1) + l];
            }
        }
    } else {
        const __half2* st = reinterpret_cast<const __half2*>(stage);
        __half* out = reinterpret_cast<__half*>(a.out);
        if (nvalid == G && KP % 8 == 0) {
            constexpr int P8 = G / 8;
            for (int idx = threadIdx.x; idx < M * 2 * P8; idx += NT) {
                const int piece = idx % P8, plane = (idx / P8) & 1, c = idx / (2 * P8);
                const uint32_t* w = reinterpret_cast<const uint32_t*>(st + c * (G + 1) + 8 * piece);
                const uint32_t sel = plane ? 0x7632u : 0x5410u;
                *reinterpret_cast<uint4*>(out + (((int64_t)c * 2 + plane) * S + s) * KP + k0 + 8 * piece) =
                    make_uint4(__byte_perm(w[0], w[1], sel), __byte_perm(w[2], w[3], sel),
                               __byte_perm(w[4], w[5], sel), __byte_perm(w[6], w[7], sel));
            }
        } else {
            for (int idx = threadIdx.x; idx < M * 2 * G; idx += NT) {
                const int l = idx % G, plane = (idx / G) & 1, c = idx / (2 * G);
                if (l < nvalid) {
                    const __half2 x = st[c * (G + 1) + l];
                    out[(((int64_t)c * 2 + plane) * S + s) * KP + k0 + l] = plane ? __high2half(x) : __low2half(x);
                }
            }
        }
    }
}

constexpr int H_G = 64, H_TP = 17, H_RAWC = 512 / 64 + 2, H_RAWW = 4 * H_RAWC;

template <int FMT>
size_t w512_smem()
{
    const size_t elem = (FMT == CS_SPECTRA_F32) ? 8 : 4;
    return (size_t)16 * 16 * H_TP * 8 + (size_t)16 * 2 * H_RAWW * 4 + 16 * 8 + (size_t)256 * (H_G + 1) * elem;
}

template <int FMT, bool PHASE>
__global__ void __launch_bounds__(256, FMT == CS_SPECTRA_F32 ? 1 : 2) k_fx_fstage_w512(const __grid_constant__ CsFStageArgs a, const float2* __restrict__ tw)
{
    constexpr int M = 256, N = 512, NT = 256, G = H_G;
    extern __shared__ __align__(16) unsigned char smem[];
    float2* tb_all = reinterpret_cast<float2*>(smem);
    uint32_t* rb_all = reinterpret_cast<uint32_t*>(tb_all + 16 * 16 * H_TP);
    float2* lut16 = reinterpret_cast<float2*>(rb_all + 16 * 2 * H_RAWW);
    unsigned char* stage = reinterpret_cast<unsigned char*>(lut16 + 16);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int hw = lane >> 4, hl = lane & 15, h = 2 * warp + hw;
    float2* tb = tb_all + h * 16 * H_TP;
    uint32_t* rb = rb_all + h * 2 * H_RAWW;
    const int s = blockIdx.y, k0 = blockIdx.x * G;
    const int64_t chunks = a.bytes_per_input >> 4;
    const unsigned char* base = a.raw + (int64_t)s * a.bytes_per_input;
    // staging column of round r: warp + 8 r', half 0 taking r' = 0, 1, 4, 5 and half 1 r' + 2
    auto slot = [&](int r) { return warp + 8 * ((r & 1) + 4 * (r >> 1) + 2 * hw); };

    auto prefetch = [&](int r) -> int {
        const int k = k0 + slot(r);
        const bool kv = k < a.K;
        const int64_t start = a.start_sample + (int64_t)k * N + ((a.shift && kv) ? __ldg(a.shift + (int64_t)s * a.K + k) : 0);
        const int64_t c0 = start >> 6;
        const uint32_t dst = (uint32_t)__cvta_generic_to_shared(rb + (r & 1) * H_RAWW);
        if (hl < H_RAWC) {
            const int64_t ci = c0 + hl;
            const bool ok = kv && ci >= 0 && ci < chunks;
            cp_async16(dst + 16 * hl, ok ? base + 16 * ci : a.raw, ok);
        }
        cp_async_commit();
        return (int)(start & 63);
    };
    int off_next = prefetch(0);

    if (threadIdx.x < 16) lut16[threadIdx.x] = make_float2(a.lut[threadIdx.x & 3], a.lut[threadIdx.x >> 2]);
    float2 w1, whalf;
    {
        float sn, cs;
        sincospif(-(float)hl / 128.0f, &sn, &cs);
        w1 = make_float2(cs, sn);                                // W_256^hl
        sincospif(-(float)hl / 256.0f, &sn, &cs);
        whalf = make_float2(0.5f * cs, 0.5f * sn);               // W_512^hl / 2
    }
    float2 wp[16];
    wp[0] = make_float2(1.f, 0.f);
    wp[1] = w1;
#pragma unroll
    for (int e = 2; e < 16; e++) wp[e] = (e & 1) ? cmul(wp[e - 1], w1) : cmul(wp[e / 2], wp[e / 2]);
    __syncthreads();
    const int src = (16 - hl) & 15;

#pragma unroll 1
    for (int r = 0; r < 4; r++) {
        const int ls = slot(r), k = k0 + ls;
        const int off = off_next;
        if (r + 1 < 4) {
            off_next = prefetch(r + 1);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncwarp();
        const uint32_t* rw = rb + (r & 1) * H_RAWW;
        const int f0 = off + 2 * hl;
        const int wb = f0 >> 4, sh = 2 * (f0 & 15);
        float2 v[16];
#pragma unroll
        for (int j = 0; j < 16; j++) {                           // pair j is 32 samples = 2 words further on
            const uint32_t bits = __funnelshift_r(rw[wb + 2 * j], rw[wb + 2 * j + 1], sh);
            v[j] = lut16[bits & 15u];
        }
        Dft<16>::run(v);
#pragma unroll
        for (int e = 1; e < 16; e++) v[e] = cmul(v[e], wp[e]);
#pragma unroll
        for (int e = 0; e < 16; e++) tb[e * H_TP + hl] = v[e];
        __syncwarp();
#pragma unroll
        for (int e = 0; e < 16; e++) v[e] = tb[hl * H_TP + e];
        __syncwarp();
        Dft<16>::run(v);                                         // v[k2] = Z[hl + 16 k2]

        // real-FFT split over the pairs (k, 256 - k), as in the 2048-point path
        const bool kv = k < a.K;
        const int64_t sk = (int64_t)s * a.K + (kv ? k : 0);
        float2 B = make_float2(1.f, 0.f), D = B, B2 = B;
        if constexpr (PHASE) {
            const float ph0 = __ldg(a.phase0 + sk), dph = __ldg(a.dphase + sk);
            float sn, cs;
            sincosf(ph0 + (float)hl * dph, &sn, &cs);
            B = make_float2(cs, sn);
            sincosf(ph0 + (float)(M - hl) * dph, &sn, &cs);
            B2 = make_float2(cs, sn);
            sincosf(16.f * dph, &sn, &cs);
            D = make_float2(cs, sn);
        }
        const float* scl = a.scale ? a.scale + (int64_t)s * M : nullptr;
        auto put = [&](int c, float2 X) {
            if (scl) X = cscale(X, __ldg(scl + c));
            if constexpr (FMT == CS_SPECTRA_F32)
                reinterpret_cast<float2*>(stage)[c * (G + 1) + ls] = X;
            else
                reinterpret_cast<__half2*>(stage)[c * (G + 1) + ls] = __floats2half2_rn(X.x, X.y);
        };
#pragma unroll
        for (int k2 = 0; k2 <= 8; k2++) {
            if (k2 == 8 && hl != 0) break;
            float2 zb;
            if (k2 < 8) {
                zb.x = __shfl_sync(0xffffffffu, v[15 - k2].x, src, 16);
                zb.y = __shfl_sync(0xffffffffu, v[15 - k2].y, src, 16);
            }
            if (hl == 0) zb = v[(16 - k2) & 15];
            const float2 za = v[k2];
            const float2 sm = make_float2(za.x + zb.x, za.y - zb.y);
            const float2 df = make_float2(za.x - zb.x, za.y + zb.y);
            const float2 t = cmul(cmul(whalf, w32(k2)), df);
            float2 X1 = make_float2(fmaf(0.5f, sm.x, t.y), fmaf(0.5f, sm.y, -t.x));
            float2 X2 = make_float2(fmaf(0.5f, sm.x, -t.y), -fmaf(0.5f, sm.y, t.x));
            const int c1 = hl + 16 * k2, c2 = M - c1;
            if constexpr (PHASE) {
                X1 = cmul(X1, B);
                X2 = cmul(X2, B2);
                B = cmul(B, D);
                B2 = cmul_conj(B2, D);
            }
            put(c1, X1);
            if (k2 < 8 && c1 != 0) put(c2, X2);
        }
    }
    __syncthreads();
    stage_writeout<FMT, M, G, NT>(a, stage, s, k0);
}

template <int FMT, bool PHASE>
int launch_w512(const CsFStageArgs& a, cudaStream_t st)
{
    const size_t smem = w512_smem<FMT>();
    auto kern = k_fx_fstage_w512<FMT, PHASE>;
    CS_CUDA_TRY(cs_smem_at_least(reinterpret_cast<const void*>(kern), (int)smem));
    kern<<<dim3((a.K + H_G - 1) / H_G, a.S), 256, smem, st>>>(a, nullptr), cs_count_launches(1);
    return (int)cudaGetLastError();
}


// ---------------------------------------------------------------------------
// N = 1024: one half-warp per segment, 32 points per lane.  The 512-point
// complex FFT is a 16 x 32 four-step: lane l keeps n = l + 16 j (j < 32),
// DFT-32 over j, twiddle W_512^(l k1), a padded 16 x 33 transpose after which
// lane l holds the 16 values of columns k1 = l and k1 = l + 16, and two
// DFT-16s give A[k2] = Z[l + 32 k2] and B[k2] = Z[l + 16 + 32 k2].  The split
// partner of Z[l + 32 k2] is Z[(32 - l) + 32 (15 - k2)], i.e. B[15 - k2] of
// lane 16 - l (lane 0: its own A[(16 - k2) mod 16]); that of Z[l + 16 + 32 k2]
// is A[15 - k2] of lane 16 - l (lane 0: its own B[15 - k2]).  CTA tiles of 64
// segments (FP16) or 32 (FP32), staged as in the 512-point form.
// ---------------------------------------------------------------------------
constexpr int Q_TP = 33, Q_RAWC = 1024 / 64 + 2, Q_RAWW = 4 * Q_RAWC;

template <int FMT>
constexpr int w1024_g() { return FMT == CS_SPECTRA_F32 ? 32 : 64; }

template <int FMT>
size_t w1024_smem()
{
    const size_t elem = (FMT == CS_SPECTRA_F32) ? 8 : 4;
    return (size_t)16 * 16 * Q_TP * 8 + (size_t)16 * 2 * Q_RAWW * 4 + 16 * 8 + (size_t)512 * (w1024_g<FMT>() + 1) * elem;
}

template <int FMT, bool PHASE>
__global__ void __launch_bounds__(256, 1) k_fx_fstage_w1024(const __grid_constant__ CsFStageArgs a, const float2* __restrict__ tw)
{
    constexpr int M = 512, N = 1024, NT = 256, G = w1024_g<FMT>(), ROUNDS = G / 16;
    extern __shared__ __align__(16) unsigned char smem[];
    float2* tb_all = reinterpret_cast<float2*>(smem);
    uint32_t* rb_all = reinterpret_cast<uint32_t*>(tb_all + 16 * 16 * Q_TP);
    float2* lut16 = reinterpret_cast<float2*>(rb_all + 16 * 2 * Q_RAWW);
    unsigned char* stage = reinterpret_cast<unsigned char*>(lut16 + 16);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int hw = lane >> 4, hl = lane & 15, h = 2 * warp + hw;
    float2* tb = tb_all + h * 16 * Q_TP;
    uint32_t* rb = rb_all + h * 2 * Q_RAWW;
    const int s = blockIdx.y, k0 = blockIdx.x * G;
    const int64_t chunks = a.bytes_per_input >> 4;
    const unsigned char* base = a.raw + (int64_t)s * a.bytes_per_input;
    // staging column of round r: the two half-warps of a warp 16 columns apart
    auto slot = [&](int r) {
        if constexpr (ROUNDS == 4) return warp + 8 * ((r & 1) + 4 * (r >> 1) + 2 * hw);
        else return warp + 8 * (r + 2 * hw);
    };

    auto prefetch = [&](int r) -> int {
        const int k = k0 + slot(r);
        const bool kv = k < a.K;
        const int64_t start = a.start_sample + (int64_t)k * N + ((a.shift && kv) ? __ldg(a.shift + (int64_t)s * a.K + k) : 0);
        const int64_t c0 = start >> 6;
        const uint32_t dst = (uint32_t)__cvta_generic_to_shared(rb + (r & 1) * Q_RAWW);
        for (int c = hl; c < Q_RAWC; c += 16) {
            const int64_t ci = c0 + c;
            const bool ok = kv && ci >= 0 && ci < chunks;
            cp_async16(dst + 16 * c, ok ? base + 16 * ci : a.raw, ok);
        }
        cp_async_commit();
        return (int)(start & 63);
    };
    int off_next = prefetch(0);

    if (threadIdx.x < 16) lut16[threadIdx.x] = make_float2(a.lut[threadIdx.x & 3], a.lut[threadIdx.x >> 2]);
    // W_512^(hl e), e < 32: e < 8 by a balanced recurrence, blocks of 8 by powers of W_512^(8 hl)
    float2 wp[8], whA, whB;
    {
        float sn, cs;
        sincospif(-(float)hl / 256.0f, &sn, &cs);
        wp[0] = make_float2(1.f, 0.f);
        wp[1] = make_float2(cs, sn);
#pragma unroll
        for (int e = 2; e < 8; e++) wp[e] = (e & 1) ? cmul(wp[e - 1], wp[1]) : cmul(wp[e / 2], wp[e / 2]);
        sincospif(-(float)hl / 512.0f, &sn, &cs);
        whA = make_float2(0.5f * cs, 0.5f * sn);                 // W_1024^hl / 2
        sincospif(-(float)(hl + 16) / 512.0f, &sn, &cs);
        whB = make_float2(0.5f * cs, 0.5f * sn);                 // W_1024^(hl + 16) / 2
    }
    const float2 w8 = cmul(wp[4], wp[4]);
    __syncthreads();
    const int src = (16 - hl) & 15;

#pragma unroll 1
    for (int r = 0; r < ROUNDS; r++) {
        const int ls = slot(r), k = k0 + ls;
        const int off = off_next;
        if (r + 1 < ROUNDS) {
            off_next = prefetch(r + 1);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncwarp();
        const uint32_t* rw = rb + (r & 1) * Q_RAWW;
        const int f0 = off + 2 * hl;
        const int wb = f0 >> 4, sh = 2 * (f0 & 15);
        float2 v[32];
#pragma unroll
        for (int j = 0; j < 32; j++) {                           // pair j is 32 samples = 2 words further on
            const uint32_t bits = __funnelshift_r(rw[wb + 2 * j], rw[wb + 2 * j + 1], sh);
            v[j] = lut16[bits & 15u];
        }
        Dft<32>::run(v);
        {
            float2 q = make_float2(1.f, 0.f);
#pragma unroll
            for (int b = 0; b < 4; b++) {
#pragma unroll
                for (int e = 0; e < 8; e++) {
                    if (b == 0 && e == 0) continue;
                    v[8 * b + e] = cmul(v[8 * b + e], b ? cmul(q, wp[e]) : wp[e]);
                }
                q = b ? cmul(q, w8) : w8;
            }
        }
#pragma unroll
        for (int e = 0; e < 32; e++) tb[hl * Q_TP + e] = v[e];
        __syncwarp();
#pragma unroll
        for (int l = 0; l < 16; l++) {
            v[l] = tb[l * Q_TP + hl];
            v[16 + l] = tb[l * Q_TP + hl + 16];
        }
        __syncwarp();
        Dft<16>::run(v);                                         // v[k2] = Z[hl + 32 k2]
        Dft<16>::run(v + 16);                                    // v[16 + k2] = Z[hl + 16 + 32 k2]

        const bool kv = k < a.K;
        const int64_t sk = (int64_t)s * a.K + (kv ? k : 0);
        float2 A1 = make_float2(1.f, 0.f), A2 = A1, B1 = A1, B2 = A1, D = A1;
        if constexpr (PHASE) {
            const float ph0 = __ldg(a.phase0 + sk), dph = __ldg(a.dphase + sk);
            float sn, cs;
            sincosf(ph0 + (float)hl * dph, &sn, &cs);            A1 = make_float2(cs, sn);
            sincosf(ph0 + (float)(M - hl) * dph, &sn, &cs);      A2 = make_float2(cs, sn);
            sincosf(ph0 + (float)(hl + 16) * dph, &sn, &cs);     B1 = make_float2(cs, sn);
            sincosf(ph0 + (float)(M - hl - 16) * dph, &sn, &cs); B2 = make_float2(cs, sn);
            sincosf(32.f * dph, &sn, &cs);                       D = make_float2(cs, sn);
        }
        const float* scl = a.scale ? a.scale + (int64_t)s * M : nullptr;
        auto put = [&](int c, float2 X) {
            if (scl) X = cscale(X, __ldg(scl + c));
            if constexpr (FMT == CS_SPECTRA_F32)
                reinterpret_cast<float2*>(stage)[c * (G + 1) + ls] = X;
            else
                reinterpret_cast<__half2*>(stage)[c * (G + 1) + ls] = __floats2half2_rn(X.x, X.y);
        };
        // X[k] = s/2 - i t, X[M - k] = conj(s/2 + i t), s = Z[k] + conj(Z[M-k]), t = (W_N^k / 2)(Z[k] - conj(Z[M-k]))
        auto split = [&](float2 za, float2 zb, float2 wh, float2& X1, float2& X2) {
            const float2 sm = make_float2(za.x + zb.x, za.y - zb.y);
            const float2 df = make_float2(za.x - zb.x, za.y + zb.y);
            const float2 t = cmul(wh, df);
            X1 = make_float2(fmaf(0.5f, sm.x, t.y), fmaf(0.5f, sm.y, -t.x));
            X2 = make_float2(fmaf(0.5f, sm.x, -t.y), -fmaf(0.5f, sm.y, t.x));
        };
#pragma unroll
        for (int k2 = 0; k2 <= 8; k2++) {
            if (k2 == 8 && hl != 0) break;
            float2 pa, pb;                                        // partners of Z[hl + 32 k2] and Z[hl + 16 + 32 k2]
            if (k2 < 8) {
                pa.x = __shfl_sync(0xffffffffu, v[16 + 15 - k2].x, src, 16);
                pa.y = __shfl_sync(0xffffffffu, v[16 + 15 - k2].y, src, 16);
                pb.x = __shfl_sync(0xffffffffu, v[15 - k2].x, src, 16);
                pb.y = __shfl_sync(0xffffffffu, v[15 - k2].y, src, 16);
            }
            if (hl == 0) {
                pa = v[(16 - k2) & 15];
                pb = v[16 + 15 - k2];
            }
            const float2 w32k = w32(k2);
            float2 X1, X2;
            split(v[k2], pa, cmul(whA, w32k), X1, X2);
            const int cA = hl + 32 * k2;
            if constexpr (PHASE) {
                X1 = cmul(X1, A1);
                X2 = cmul(X2, A2);
                A1 = cmul(A1, D);
                A2 = cmul_conj(A2, D);
            }
            put(cA, X1);
            if (k2 < 8 && cA != 0) put(M - cA, X2);
            if (k2 < 8) {
                split(v[16 + k2], pb, cmul(whB, w32k), X1, X2);
                const int cB = hl + 16 + 32 * k2;
                if constexpr (PHASE) {
                    X1 = cmul(X1, B1);
                    X2 = cmul(X2, B2);
                    B1 = cmul(B1, D);
                    B2 = cmul_conj(B2, D);
                }
                put(cB, X1);
                put(M - cB, X2);
            }
        }
    }
    __syncthreads();
    stage_writeout<FMT, M, G, NT>(a, stage, s, k0);
}

template <int FMT, bool PHASE>
int launch_w1024(const CsFStageArgs& a, cudaStream_t st)
{
    const size_t smem = w1024_smem<FMT>();
    auto kern = k_fx_fstage_w1024<FMT, PHASE>;
    CS_CUDA_TRY(cs_smem_at_least(reinterpret_cast<const void*>(kern), (int)smem));
    constexpr int G = w1024_g<FMT>();
    kern<<<dim3((a.K + G - 1) / G, a.S), 256, smem, st>>>(a, nullptr), cs_count_launches(1);
    return (int)cudaGetLastError();
}

}  // namespace

void cs_fstage_allow_timing(bool allow) { t_w2048_timing_allowed = allow; }
bool cs_fstage_timing_allowed() { return t_w2048_timing_allowed; }

namespace {

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

bool cs_fstage_kblocked(const CsFStageArgs& a)
{
    const int kp = a.kp ? a.kp : a.K;
    if (cs_fstage_tc_supported(a)) {             // the opt-in tensor-core F stage writes the planes
        const char* e = getenv("CELLSPE_FSTAGE_TC");
        if (e && e[0] == '1') return false;
    }
    return a.format == CS_SPECTRA_F16 && a.N == 2048 && !a.msb_first && !a.seg_major && a.K % 32 == 0 &&
           kp % 32 == 0;
}

int cs_fstage_layout(const CsFStageArgs& a)
{
    if (!cs_fstage_kblocked(a)) return 0;
    CsFStageArgs k = a;
    k.kblock = 1;
    if (!cs_fstage_tc32_supported(k)) return 1;
    const char* e = getenv("CELLSPE_FSTAGE_TC32");
    return e && (e[0] == '0' || e[0] == '1') ? 1 : 2;
}

int cs_fx_fstage(const CsFStageArgs& a, cudaStream_t st)
{
    if (!a.raw || !a.out || a.S <= 0 || a.K <= 0) return CS_ERR_ARG;
    if ((uintptr_t)a.raw % 16 || a.bytes_per_input % 16 || (uintptr_t)a.out % 16) return CS_ERR_ARG;
    if (a.kblock < 0 || a.kblock > 2 || (a.kblock && !cs_fstage_kblocked(a))) return CS_ERR_ARG;
    // channel-grouped k-blocked spectra: only the warp-specialised form writes them
    if (a.kblock == 2) return cs_fstage_tc32_supported(a) ? cs_fx_fstage_tc32(a, st, true) : CS_ERR_ARG;
    // The tensor-core F stage is opt-in (CELLSPE_FSTAGE_TC=1, read per call):
    // its 8-segment units give 16-byte output runs, and on 512 inputs x 4096
    // segments it measured 14.5 ms against 7.3 ms for the 16-segment warp
    // FFT below.  It writes the channel-major planes only.
    if (!a.kblock && cs_fstage_tc_supported(a)) {
        const char* e = getenv("CELLSPE_FSTAGE_TC");
        if (e && e[0] == '1') return cs_fx_fstage_tc(a, st);
    }
    // N = 2048 k-blocked FP16 spectra (layout 1): the lockstep tensor-core
    // form when CELLSPE_FSTAGE_TC32=1 (read per call), else the warp FFT below.
    // (The warp-specialised form, the default, writes layout 2 above.)
    if (a.kblock == 1 && cs_fstage_tc32_supported(a)) {
        const char* e = getenv("CELLSPE_FSTAGE_TC32");
        if (e && e[0] == '1') return cs_fx_fstage_tc32(a, st, false);
    }
    if (a.N == 2048 && !a.msb_first) {
        const bool ph = a.phase0 != nullptr;
        if (a.format == CS_SPECTRA_F32)
            return ph ? launch_w2048<CS_SPECTRA_F32, true>(a, st) : launch_w2048<CS_SPECTRA_F32, false>(a, st);
        return ph ? launch_w2048<CS_SPECTRA_F16, true>(a, st) : launch_w2048<CS_SPECTRA_F16, false>(a, st);
    }
    // N = 512, 1024 (channel-major) and N = 4096 ... 32768 (segment-major): the
    // warp four-steps (CELLSPE_FSTAGE_GENERIC=1 selects the CTA-wide Stockham FFT)
    const char* gen = getenv("CELLSPE_FSTAGE_GENERIC");
    const bool generic = gen && gen[0] == '1';
    if (a.N == 512 && !a.seg_major && !a.msb_first && !generic) {
        const bool ph = a.phase0 != nullptr;
        if (a.format == CS_SPECTRA_F32)
            return ph ? launch_w512<CS_SPECTRA_F32, true>(a, st) : launch_w512<CS_SPECTRA_F32, false>(a, st);
        return ph ? launch_w512<CS_SPECTRA_F16, true>(a, st) : launch_w512<CS_SPECTRA_F16, false>(a, st);
    }
    if (a.N == 1024 && !a.seg_major && !a.msb_first && !generic) {
        const bool ph = a.phase0 != nullptr;
        if (a.format == CS_SPECTRA_F32)
            return ph ? launch_w1024<CS_SPECTRA_F32, true>(a, st) : launch_w1024<CS_SPECTRA_F32, false>(a, st);
        return ph ? launch_w1024<CS_SPECTRA_F16, true>(a, st) : launch_w1024<CS_SPECTRA_F16, false>(a, st);
    }
    if (a.seg_major && !a.msb_first && a.N >= 4096 && a.N <= 32768) {
        if (!generic) {
            switch (a.N) {
                case 4096: return dispatch_wbig<2>(a, st);
                case 8192: return dispatch_wbig<4>(a, st);
                case 16384: return dispatch_wbig<8>(a, st);
                default: return dispatch_wbig<16>(a, st);
            }
        }
    }
    switch (a.N) {
        case 512: return dispatch_fstage<256>(a, st);
        case 1024: return dispatch_fstage<512>(a, st);
        case 2048: return dispatch_fstage<1024>(a, st);
        case 4096: return dispatch_fstage<2048>(a, st);
        case 8192: return dispatch_fstage<4096>(a, st);
        case 16384: return dispatch_fstage<8192>(a, st);
        case 32768: return dispatch_fstage<16384>(a, st);
        default: return CS_ERR_UNSUPPORTED;
    }
}

namespace {

// [S][K][C] -> channel-major rows.  Tile of 64 segments x 64 channels per
// CTA: 256-byte reads along channels, 128- (F16) or 512-byte (F32) writes
// along segments.
constexpr int TT = 64;

__global__ void __launch_bounds__(256) k_transpose_f16(const __half2* __restrict__ in, int K, int C, int kp, int S_out,
                                                       __half* __restrict__ out, int vec)
{
    __shared__ uint32_t tile[TT][TT + 1];            // half2 bits; the odd row stride keeps both passes conflict-free
    const int s = blockIdx.z, k0 = blockIdx.y * TT, c0 = blockIdx.x * TT;
    // vec: 16-byte aligned rows in and out (C % 4 == 0, kp % 8 == 0, aligned bases)
    const bool full = vec && k0 + TT <= K && c0 + TT <= C;
    if (full) {
        // 64 rows x 16 uint4 (4 channels each)
        for (int i = threadIdx.x; i < TT * (TT / 4); i += 256) {
            const int kk = i / (TT / 4), q = i % (TT / 4);
            const uint4 v = *reinterpret_cast<const uint4*>(in + ((int64_t)s * K + k0 + kk) * C + c0 + 4 * q);
            tile[kk][4 * q] = v.x;
            tile[kk][4 * q + 1] = v.y;
            tile[kk][4 * q + 2] = v.z;
            tile[kk][4 * q + 3] = v.w;
        }
    } else {
        for (int i = threadIdx.x; i < TT * TT; i += 256) {
            const int kk = i / TT, cc = i % TT, k = k0 + kk, c = c0 + cc;
            const __half2 x = (k < K && c < C) ? in[((int64_t)s * K + k) * C + c] : __floats2half2_rn(0.f, 0.f);
            tile[kk][cc] = *reinterpret_cast<const uint32_t*>(&x);
        }
    }
    __syncthreads();
    if (full) {
        // rows (c, plane) of 64 halves as 8 pieces of 16 bytes: the Re (low) or
        // Im (high) halves of 8 consecutive segments
        for (int i = threadIdx.x; i < TT * 2 * (TT / 8); i += 256) {
            const int pc = i % (TT / 8), row = i / (TT / 8), cc = row >> 1, plane = row & 1;
            uint32_t w[8];
#pragma unroll
            for (int j = 0; j < 8; j++) w[j] = tile[8 * pc + j][cc];
            const uint32_t sel = plane ? 0x7632u : 0x5410u;
            *reinterpret_cast<uint4*>(out + (((int64_t)(c0 + cc) * 2 + plane) * S_out + s) * kp + k0 + 8 * pc) =
                make_uint4(__byte_perm(w[0], w[1], sel), __byte_perm(w[2], w[3], sel), __byte_perm(w[4], w[5], sel),
                           __byte_perm(w[6], w[7], sel));
        }
        return;
    }
    // row (c, plane): 64 halves of k as 32 half pairs
    for (int i = threadIdx.x; i < TT * 2 * (TT / 2); i += 256) {
        const int w = i % (TT / 2), row = i / (TT / 2), cc = row >> 1, plane = row & 1;
        const int c = c0 + cc, k = k0 + 2 * w;
        if (c >= C || k >= K) continue;
        const uint32_t a = tile[2 * w][cc], b = tile[2 * w + 1][cc];
        __half* o = out + (((int64_t)c * 2 + plane) * S_out + s) * kp + k;
        if (k + 1 < K) {
            *reinterpret_cast<uint32_t*>(o) = __byte_perm(a, b, plane ? 0x7632u : 0x5410u);
        } else {
            const uint32_t h = plane ? (a >> 16) : (a & 0xFFFFu);
            *reinterpret_cast<unsigned short*>(o) = (unsigned short)h;
        }
    }
}

__global__ void __launch_bounds__(256) k_transpose_f32(const float2* __restrict__ in, int K, int C, int kp, int S_out,
                                                       float2* __restrict__ out)
{
    __shared__ float2 tile[TT][TT + 1];
    const int s = blockIdx.z, k0 = blockIdx.y * TT, c0 = blockIdx.x * TT;
    for (int i = threadIdx.x; i < TT * TT; i += 256) {
        const int kk = i / TT, cc = i % TT, k = k0 + kk, c = c0 + cc;
        tile[kk][cc] = (k < K && c < C) ? in[((int64_t)s * K + k) * C + c] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < TT * TT; i += 256) {
        const int kk = i % TT, cc = i / TT, c = c0 + cc, k = k0 + kk;
        if (c < C && k < K) out[((int64_t)c * S_out + s) * kp + k] = tile[kk][cc];
    }
}

}  // namespace

int cs_spectra_transpose(const void* tmp, int S, int K, int C, int kp, int S_out, int format, void* out, cudaStream_t st)
{
    if (!tmp || !out || S <= 0 || K <= 0 || C <= 0 || kp < K || S_out < S || S > 65535) return CS_ERR_ARG;
    const dim3 grid((C + TT - 1) / TT, (K + TT - 1) / TT, S);
    if (grid.y > 65535) return CS_ERR_ARG;
    if (format == CS_SPECTRA_F32) {
        k_transpose_f32<<<grid, 256, 0, st>>>((const float2*)tmp, K, C, kp, S_out, (float2*)out), cs_count_launches(1);
    } else {
        if ((uintptr_t)out % 4 || kp % 2) return CS_ERR_ARG;
        const int vec = (C % 4 == 0 && kp % 8 == 0 && (uintptr_t)tmp % 16 == 0 && (uintptr_t)out % 16 == 0) ? 1 : 0;
        k_transpose_f16<<<grid, 256, 0, st>>>((const __half2*)tmp, K, C, kp, S_out, (__half*)out, vec),
            cs_count_launches(1);
    }
    return (int)cudaGetLastError();
}
