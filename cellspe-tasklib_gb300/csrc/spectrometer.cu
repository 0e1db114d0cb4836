// K-e + K-pcal: spectrometer power accumulation and phase-cal extraction.
//
// Semantics (TaskCoreIPP::doMaths, spectrometer/src/IA-32/TaskCoreIPP.cpp:
// 394-513, one source per subband): spectrum `spec` of subband `sub` is built
// from novl = overlap*K - (overlap-1) FFTs (swspectrometer.cpp:231) that start
// every N/overlap samples from sample spec*K*N; each FFT windows N samples
// (generate_windowfunction :569-605), takes the real FFT, and adds |X_k|^2 for
// k = 1..N/2-1 and X_0^2, X_{N/2}^2 (DC and Nyquist real, :437-447); the sum
// is scaled by 1/novl (:124, :493).
//
// GPU layout: the CTA grid is (chunk of CH FFTs) x (subband, spectrum) x
// (split p).  Inside a CTA, groups of M/16 threads run CtaFft on different
// FFTs of the chunk and accumulate |X|^2 into thread-owned shared-memory bins;
// the CTA writes one partial spectrum per chunk to scratch, and a reduce
// kernel adds the partials in chunk order (deterministic) and applies 1/novl.
// N = 65536 does not fit one SM's shared memory (32768 complex points), so it
// is split across two CTAs by output parity: CTA p computes the M/2-point FFT
// of y_p[n] = (z[n] + (-1)^p z[n + M/2]) W_M^{n p}, which yields
// Z[2m + p]; the real-FFT pairs (k, M-k) keep the parity, so each CTA finishes
// its own bins without exchanging data (input words are read twice, at 0.25 B
// per sample).
//
// Phase-cal (TaskCoreIPP::extract_PCal :633-693, settings
// swspectrometer.cpp:180-184): on the non-overlapped FFTs (every overlap-th),
// i.e. on every sample of the spectrum once, bins[(n mod L) mod T] +=
// x[n] * exp(-2 pi i f_off (n mod L) / fs), L = rotator length, T = tone
// bins.  Tones = DFT(bins)/T, first ntones (PCal.cpp:280-300, getFinalPCal).
#include "common.cuh"
#include "kernels.h"

#include <cmath>
#include <cstdlib>
#include <map>
#include <mutex>
#include <type_traits>
#include <vector>

namespace {

constexpr int SPEC_CH = 32;   // FFTs per chunk (one partial spectrum each)

template <int MC> struct SCfg {
    static constexpr int T = MC / 16;
    static constexpr int GROUPS = (T >= 256) ? 1 : 256 / T;
    static constexpr int NT = T * GROUPS;
};

std::mutex g_win_mu;
std::map<std::tuple<int, int, int>, float*> g_win;   // (device, type, n)

const float* window_table(int type, int n)
{
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(g_win_mu);
    auto key = std::make_tuple(dev, type, n);
    auto it = g_win.find(key);
    if (it != g_win.end()) return it->second;
    std::vector<float> h(n);
    for (int i = 0; i < n; i++) h[i] = (float)cs_window_value(type, i, n);
    float* d = nullptr;
    if (cudaMalloc(&d, sizeof(float) * n) != cudaSuccess) return nullptr;
    cudaMemcpy(d, h.data(), sizeof(float) * n, cudaMemcpyHostToDevice);
    g_win[key] = d;
    return d;
}

std::map<std::tuple<int, int, long long, long long>, float2*> g_rot;

const float2* rotator_table(int L, double off_hz, double fs_hz)
{
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(g_win_mu);
    auto key = std::make_tuple(dev, L, (long long)llround(off_hz * 1e3), (long long)llround(fs_hz));
    auto it = g_rot.find(key);
    if (it != g_rot.end()) return it->second;
    std::vector<float2> h(L);
    double dphi = 2 * M_PI * (-off_hz / fs_hz);
    for (int i = 0; i < L; i++) h[i] = make_float2((float)std::cos(dphi * i), (float)std::sin(dphi * i));
    float2* d = nullptr;
    if (cudaMalloc(&d, sizeof(float2) * L) != cudaSuccess) return nullptr;
    cudaMemcpy(d, h.data(), sizeof(float2) * L, cudaMemcpyHostToDevice);
    g_rot[key] = d;
    return d;
}

CS_DEV float lut_pick4(const float (&l)[4], unsigned c)
{
    float lo = (c & 1u) ? l[1] : l[0];
    float hi = (c & 1u) ? l[3] : l[2];
    return (c & 2u) ? hi : lo;
}

// Samples s and s+1 (s even) of a plane word through a 16-entry table of
// level pairs (one shared-memory read instead of two 4-way selects); blanked
// samples (their bit in the validity mask clear) are 0.0, as mark5access
// decodes them.
CS_DEV float2 sample_pair16(const float2* __restrict__ lut16, uint32_t w, int f, const uint32_t* __restrict__ vmask,
                            int64_t s)
{
    float2 x = lut16[(w >> (2 * f)) & 15u];
    if (vmask) {
        const uint32_t m = __ldg(vmask + (s >> 5)) >> (s & 31);
        x.x = (m & 1u) ? x.x : 0.f;
        x.y = (m & 2u) ? x.y : 0.f;
    }
    return x;
}

template <int MC, int P>
__global__ void __launch_bounds__(SCfg<MC>::NT) k_spec_power(const __grid_constant__ CsSpecArgs a, const float2* __restrict__ tw,
                                                            const float* __restrict__ win, int nchunk, int ch)
{
    using C = SCfg<MC>;
    constexpr int T = C::T, GROUPS = C::GROUPS;
    constexpr int M = MC * P, N = 2 * M;
    constexpr int NACC = M / P + 1;                 // owned bins (local index)
    extern __shared__ __align__(16) unsigned char smem[];
    float2* fb_all = reinterpret_cast<float2*>(smem);
    float* acc_all = reinterpret_cast<float*>(fb_all + GROUPS * fpad_size(MC));

    const int g = threadIdx.x / T, t = threadIdx.x % T;
    float2* fb = fb_all + g * fpad_size(MC);
    float* acc = acc_all + g * NACC;
    const int chunk = blockIdx.x;
    const int row = blockIdx.y;                      // sub * nspec + spec
    const int sub = row / a.nspec, spec = row % a.nspec;
    const int p = (P == 2) ? (int)blockIdx.z : 0;
    const int novl = a.overlap * a.ffts_per_spectrum - (a.overlap - 1);
    const int hop = N / a.overlap;
    const uint32_t* plane = reinterpret_cast<const uint32_t*>(a.planes + (int64_t)sub * a.bytes_per_sub);
    const float lut[4] = {a.lut[0], a.lut[1], a.lut[2], a.lut[3]};
    const uint32_t* vmask = a.valid_mask;

    __shared__ float2 lut16[16];                     // level pairs: entry bits = code0 + 4 code1
    if (threadIdx.x < 16) lut16[threadIdx.x] = make_float2(lut[threadIdx.x & 3], lut[threadIdx.x >> 2]);
    for (int i = threadIdx.x; i < GROUPS * NACC; i += C::NT) acc_all[i] = 0.f;
    __syncthreads();

    const int j_begin = chunk * ch, j_end = min(novl, j_begin + ch);
    auto bar = [] { __syncthreads(); };
    // P = 2, odd outputs: sample pair n = t + r T is rotated by W_N^(2n) =
    // W_N^(2t) W_32^r (2T = N/32), one table load for all windows
    const float2 tw_t = (P == 2) ? twiddle(tw, 2 * t) : make_float2(1.f, 0.f);
    for (int j0 = j_begin; j0 < j_end; j0 += GROUPS) {
        const int j = j0 + g;
        const bool valid = j < j_end;
        const int64_t start = (int64_t)spec * a.ffts_per_spectrum * N + (int64_t)(valid ? j : j_begin) * hop;
        const uint32_t* wsrc = plane + (start >> 4);
        float2 v[16];
#pragma unroll
        for (int r = 0; r < 16; r++) {
            const int n = t + r * T;                 // index into the transformed sequence
            // window values of samples 2n, 2n+1 as one 8-byte load
            const float2* win2 = reinterpret_cast<const float2*>(win);
            if constexpr (P == 1) {
                uint32_t w = __ldg(wsrc + (2 * n >> 4));
                int f = (2 * n) & 15;
                const float2 x = sample_pair16(lut16, w, f, vmask, start + 2 * n);
                const float2 wn = __ldg(win2 + n);
                v[r] = make_float2(x.x * wn.x, x.y * wn.y);
            } else {
                const int n2 = n + MC;
                uint32_t w1 = __ldg(wsrc + (2 * n >> 4)), w2 = __ldg(wsrc + (2 * n2 >> 4));
                int f1 = (2 * n) & 15, f2 = (2 * n2) & 15;
                const float2 x1 = sample_pair16(lut16, w1, f1, vmask, start + 2 * n);
                const float2 x2 = sample_pair16(lut16, w2, f2, vmask, start + 2 * n2);
                // cosine^2: w(i + N/2) = sin^2 = 1 - w(i), so one table read
                // serves both halves (the table pair differs by <= 2^-24)
                const float2 wa = __ldg(win2 + n);
                const float2 wb = (a.window == 2) ? make_float2(1.f - wa.x, 1.f - wa.y) : __ldg(win2 + n2);
                float2 z1 = make_float2(x1.x * wa.x, x1.y * wa.y);
                float2 z2 = make_float2(x2.x * wb.x, x2.y * wb.y);
                v[r] = p ? cmul(csub(z1, z2), rot32(tw_t, r)) : cadd(z1, z2);
            }
        }
        CtaFft<MC, (MC >= 2048)>::run(fb, t, v, tw, N / MC, bar);
        if (valid) {
            const int mmax = (P == 1) ? MC / 2 : (p ? MC / 2 - 1 : MC / 2);
            for (int m = t; m <= mmax; m += T) {
                int k = P * m + p;
                int mb = (P == 1 || p == 0) ? ((MC - m) & (MC - 1)) : (MC - 1 - m);
                float2 Xk, Xm;
                r2c_pair(fb[fpad(m)], fb[fpad(mb)], twiddle(tw, k), Xk, Xm);
                if (k == 0) {
                    acc[0] += Xk.x * Xk.x;
                    acc[M / P] += Xm.x * Xm.x;
                } else {
                    acc[k / P] += Xk.x * Xk.x + Xk.y * Xk.y;
                    if (k != M / 2) acc[(M - k) / P] += Xm.x * Xm.x + Xm.y * Xm.y;
                }
            }
        }
        bar();
    }
    // combine groups, write the chunk partial (owned bins only)
    float* prow = a.partial + ((int64_t)row * nchunk + chunk) * (M + 1);
    for (int l = threadIdx.x; l < NACC; l += C::NT) {
        int k = P * l + p;
        if (k > M) continue;
        float s = 0.f;
#pragma unroll
        for (int gg = 0; gg < GROUPS; gg++) s += acc_all[gg * NACC + l];
        prow[k] = s;
    }
}

// N = 32768 (P = 1) and 65536 (P = 2): the CTA's 16384-point complex FFT as
// a warp four-step with decimation in frequency, so that every input read
// (plane words, window pairs, twiddles) is coalesced across threads:
//   n = 1024 n1 + m (n1 < 16, m < 1024),  k = k1 + 16 k2 (k1 < 16, k2 < 1024)
//   W_MC^(n k) = W_16^(n1 k1) W_MC^(m k1) W_1024^(m k2).
// Column phase: thread t takes columns m = t, t + 512: 16 windowed inputs
// (P = 2: the parity fold of both halves), DFT-16 over n1, twiddle
// W_MC^(m k1), stored to row k1 of a [16][1088] tile.  Row phase: warp k1
// takes row k1: a 1024-point DFT in registers (32 points per lane: DFT-32,
// twiddle, transpose through the row's own padded region, DFT-32) and stores
// Y[k1][k2] back in natural k2 order.  Pair phase: each thread owns fixed
// items (k1, k2) whose real-FFT partner lies in row 16 - k1 (P = 1 and p = 0)
// or 15 - k1 (p = 1), splits them (r2c_pair) and adds |X|^2 into its own
// shared-memory slots [slot][thread] (no two threads share a bin), which the
// CTA writes as the chunk's partial spectrum.  512 threads, one CTA per SM.
constexpr int SW_NT = 512, SW_MC = 16384, SW_ROWP = 1088, SW_SLOTS = 34;

// tile column of index k2 (or m): two float2 of padding after every 32
CS_DEV int sw_pad(int k2) { return k2 + 2 * (k2 >> 5); }

template <int P, bool MASK>
__global__ void __launch_bounds__(SW_NT, 1) k_spec_power_w(const __grid_constant__ CsSpecArgs a, const float2* __restrict__ tw,
                                                           const float* __restrict__ win, int nchunk, int ch)
{
    constexpr int MC = SW_MC, M = MC * P, N = 2 * M;
    extern __shared__ __align__(16) unsigned char smem[];
    float2* tile = reinterpret_cast<float2*>(smem);                       // [16][SW_ROWP]
    float* slots = reinterpret_cast<float*>(tile + 16 * SW_ROWP);         // [SW_SLOTS][SW_NT]
    uint32_t* rawsm = reinterpret_cast<uint32_t*>(slots + SW_SLOTS * SW_NT);   // the FFT's N / 16 plane words
    __shared__ float2 lut16[16];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int chunk = blockIdx.x, row = blockIdx.y;
    const int sub = row / a.nspec, spec = row % a.nspec;
    const int p = (P == 2) ? (int)blockIdx.z : 0;
    const int novl = a.overlap * a.ffts_per_spectrum - (a.overlap - 1);
    const int hop = N / a.overlap;
    const uint32_t* plane = reinterpret_cast<const uint32_t*>(a.planes + (int64_t)sub * a.bytes_per_sub);
    // blanking mask only in the MASK form (framed recordings), so the plain
    // form carries no per-sample mask code
    const uint32_t* vmask = MASK ? a.valid_mask : nullptr;
    const float2* win2 = reinterpret_cast<const float2*>(win);
    if (tid < 16) lut16[tid] = make_float2(a.lut[tid & 3], a.lut[tid >> 2]);
    for (int i = tid; i < SW_SLOTS * SW_NT; i += SW_NT) slots[i] = 0.f;

    // pair items of this thread: (k1, k2) with partner (k1', k2')
    //  P = 1 / p = 0: rows 1..7 (k2 = t, t + 512), row 8 (k2 = t), row 0 (k2 = t; t = 0 also k2 = 512)
    //  p = 1:         rows 0..7 (k2 = t, t + 512)
    const bool odd = P == 2 && p == 1;
    // row-phase twiddles W_1024^(lane e), e < 8 (balanced recurrence), and
    // W_1024^(8 lane), kept in shared memory [e][lane] for every warp
    __shared__ float2 wps[9][32];
    if (warp == 0) {
        float2 wp[8];
        float sn, cs;
        sincospif(-(float)lane / 512.0f, &sn, &cs);
        wp[0] = make_float2(1.f, 0.f);
        wp[1] = make_float2(cs, sn);
#pragma unroll
        for (int e = 2; e < 8; e++) wp[e] = (e & 1) ? cmul(wp[e - 1], wp[1]) : cmul(wp[e / 2], wp[e / 2]);
#pragma unroll
        for (int e = 0; e < 8; e++) wps[e][lane] = wp[e];
        wps[8][lane] = cmul(wp[4], wp[4]);
    }
    // per-thread constants: W_M^m and W_MC^m of the thread's two columns m = t, t + 512;
    // the split twiddle W_N^k of item (k1, k2), k = P (k1 + 16 k2) + p, as
    // ck[k1] = W_N^(P k1 + p) (shared, broadcast) times W_N^(16 P k2) of k2 = t, t + 512
    __shared__ float2 ck[16];
    if (tid < 16) ck[tid] = __ldg(tw + P * tid + p);
    float2 tmc[2], umc[2], bk[2];
#pragma unroll
    for (int c = 0; c < 2; c++) {
        const int m = tid + SW_NT * c;                   // column-phase columns and pair-phase k2
        tmc[c] = (P == 2) ? __ldg(tw + 2 * m) : make_float2(1.f, 0.f);   // W_M^m
        umc[c] = __ldg(tw + 2 * P * m);                  // W_MC^m
        bk[c] = __ldg(tw + 16 * P * m);                  // W_N^(16 P k2)
    }
    const float2 bk512 = __ldg(tw + 16 * P * 512);       // k2 = 512 (thread 0's extra item)
    __syncthreads();

    const int j_begin = chunk * ch, j_end = min(novl, j_begin + ch);
    // the plane words of FFT j go to shared memory by cp.async (hop is a
    // multiple of 64 samples, so each FFT starts on a 16-byte boundary); the
    // next FFT's are fetched while this one's row and pair phases run
    auto fetch = [&](int jj) {
        const int64_t st = (int64_t)spec * a.ffts_per_spectrum * N + (int64_t)jj * hop;
        const char* src = reinterpret_cast<const char*>(plane + (st >> 4));
        const uint32_t dst = (uint32_t)__cvta_generic_to_shared(rawsm);
        for (int i = tid; i < N / 64; i += SW_NT)
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst + 16 * i), "l"(src + 16 * i) : "memory");
        asm volatile("cp.async.commit_group;" ::: "memory");
    };
    if (j_begin < j_end) fetch(j_begin);
    for (int j = j_begin; j < j_end; j++) {
        const int64_t start = (int64_t)spec * a.ffts_per_spectrum * N + (int64_t)j * hop;   // a multiple of 64
        const uint32_t* wsrc = rawsm;
        asm volatile("cp.async.wait_group 0;" ::: "memory");
        __syncthreads();                                   // this FFT's words are in
        // ---- column phase: columns m = t, t + 512 ----
        // (the mask is applied only to windows that contain blanked samples)
        auto column_phase = [&](auto masked) {
        const uint32_t* vm = decltype(masked)::value ? vmask : nullptr;
#pragma unroll 1
        for (int c = 0; c < 2; c++) {
            const int m = tid + SW_NT * c;
            float2 v[16];
            const float2 tm = c ? tmc[1] : tmc[0];                                     // W_M^m
#pragma unroll
            for (int n1 = 0; n1 < 16; n1++) {
                const int n = 1024 * n1 + m;
                const float2 x1 = sample_pair16(lut16, wsrc[n >> 3], (2 * n) & 15, vm, start + 2 * n);
                const float2 wa = __ldg(win2 + n);
                const float2 z1 = make_float2(x1.x * wa.x, x1.y * wa.y);
                if constexpr (P == 1) {
                    v[n1] = z1;
                } else {
                    const int n2 = n + MC;
                    const float2 x2 = sample_pair16(lut16, wsrc[n2 >> 3], (2 * n2) & 15, vm, start + 2 * n2);
                    // cosine^2: w(i + N/2) = 1 - w(i) (one table read for both halves)
                    const float2 wb = (a.window == 2) ? make_float2(1.f - wa.x, 1.f - wa.y) : __ldg(win2 + n2);
                    const float2 z2 = make_float2(x2.x * wb.x, x2.y * wb.y);
                    // y_1[n] = (z[n] - z[n + MC]) W_M^n, W_M^(1024 n1 + m) = W_32^n1 W_M^m
                    v[n1] = p ? cmul(csub(z1, z2), rot32(tm, n1)) : cadd(z1, z2);
                }
            }
            Dft<16>::run(v);
            // W_MC^(m k1): powers of u = W_MC^m by a balanced recurrence
            const float2 u = c ? umc[1] : umc[0];
            float2 wk[16];
            wk[0] = make_float2(1.f, 0.f);
            wk[1] = u;
#pragma unroll
            for (int e = 2; e < 16; e++) wk[e] = (e & 1) ? cmul(wk[e - 1], u) : cmul(wk[e / 2], wk[e / 2]);
#pragma unroll
            for (int k1 = 0; k1 < 16; k1++) tile[k1 * SW_ROWP + sw_pad(m)] = k1 ? cmul(v[k1], wk[k1]) : v[k1];
        }
        };
        bool blanked = false;
        if constexpr (MASK) {
            // any blanked sample in this window? (N / 32 mask words, a few per thread)
            const uint32_t* mw = vmask + (start >> 5);
            bool mine = false;
            for (int i = tid; i < N / 32; i += SW_NT) mine |= __ldg(mw + i) != 0xffffffffu;
            blanked = __syncthreads_or(mine) != 0;
        }
        if (blanked) column_phase(std::true_type{});
        else column_phase(std::false_type{});
        __syncthreads();                                   // the words are consumed: fetch the next FFT's
        if (j + 1 < j_end) fetch(j + 1);
        // ---- row phase: warp k1 ----
        {
            float2* rowp = tile + warp * SW_ROWP;
            float2 x[32];
#pragma unroll
            for (int e = 0; e < 32; e++) x[e] = rowp[lane + 34 * e];          // m = lane + 32 e
            Dft<32>::run(x);
            float2 q = make_float2(1.f, 0.f);
            const float2 w8 = wps[8][lane];
#pragma unroll
            for (int b = 0; b < 4; b++) {
#pragma unroll
                for (int r = 0; r < 8; r++) {
                    if (b == 0 && r == 0) continue;
                    const float2 wr = wps[r][lane];
                    x[8 * b + r] = cmul(x[8 * b + r], b ? cmul(q, wr) : wr);
                }
                q = b ? cmul(q, w8) : w8;
            }
            __syncwarp();
#pragma unroll
            for (int e = 0; e < 32; e++) rowp[e * 33 + lane] = x[e];
            __syncwarp();
#pragma unroll
            for (int e = 0; e < 32; e++) x[e] = rowp[lane * 33 + e];
            Dft<32>::run(x);                                                    // x[e] = Y[warp][lane + 32 e]
            __syncwarp();
#pragma unroll
            for (int e = 0; e < 32; e++) rowp[lane + 34 * e] = x[e];          // k2 = lane + 32 e
        }
        __syncthreads();
        // ---- pair phase ----
        int s = 0;
        // SPECIAL: row 0 of the even forms, which holds k = 0 (DC and Nyquist
        // from Z[0]) and k = M/2 (its own partner)
        auto item = [&](int k1, int k2, float2 b, bool special) {
            int k1b, k2b;
            if (odd) k1b = 15 - k1, k2b = 1023 - k2;
            else if (k1 == 0) k1b = 0, k2b = (1024 - k2) & 1023;
            else k1b = 16 - k1, k2b = 1023 - k2;
            const float2 za = tile[k1 * SW_ROWP + sw_pad(k2)], zb = tile[k1b * SW_ROWP + sw_pad(k2b)];
            const int mp = k1 + 16 * k2;                   // index in the CTA's transform
            const int k = P * mp + p;                      // bin of the full real FFT
            float2 Xk, Xm;
            r2c_pair(za, zb, cmul(ck[k1], b), Xk, Xm);          // W_N^k
            if (special && k == 0) {
                slots[s * SW_NT + tid] += Xk.x * Xk.x;
                slots[(s + 1) * SW_NT + tid] += Xm.x * Xm.x;
            } else {
                slots[s * SW_NT + tid] += Xk.x * Xk.x + Xk.y * Xk.y;
                if (!special || k != M / 2) slots[(s + 1) * SW_NT + tid] += Xm.x * Xm.x + Xm.y * Xm.y;
            }
            s += 2;
        };
        if (odd) {
#pragma unroll
            for (int k1 = 0; k1 < 8; k1++) item(k1, tid, bk[0], false), item(k1, tid + SW_NT, bk[1], false);
        } else {
#pragma unroll
            for (int k1 = 1; k1 < 8; k1++) item(k1, tid, bk[0], false), item(k1, tid + SW_NT, bk[1], false);
            item(8, tid, bk[0], false);
            item(0, tid, bk[0], true);
            if (tid == 0) item(0, 512, bk512, true);
        }
        __syncthreads();                                   // the tile is rewritten by the next FFT
    }
    // ---- the chunk's partial spectrum: the same items' bins ----
    float* prow = a.partial + ((int64_t)row * nchunk + chunk) * (M + 1);
    int s = 0;
    auto put = [&](int k1, int k2) {
        const int k = P * (k1 + 16 * k2) + p;
        if (k == 0) {
            prow[0] = slots[s * SW_NT + tid];
            prow[M] = slots[(s + 1) * SW_NT + tid];
        } else {
            prow[k] = slots[s * SW_NT + tid];
            if (k != M / 2) prow[M - k] = slots[(s + 1) * SW_NT + tid];
        }
        s += 2;
    };
    if (odd) {
        for (int k1 = 0; k1 < 8; k1++) put(k1, tid), put(k1, tid + SW_NT);
    } else {
        for (int k1 = 1; k1 < 8; k1++) put(k1, tid), put(k1, tid + SW_NT);
        put(8, tid);
        put(0, tid);
        if (tid == 0) put(0, 512);
    }
}

__global__ void k_spec_reduce(const float* __restrict__ partial, float* __restrict__ power, int rows, int nchunk,
                              int nb, float scale)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)rows * nb) return;
    int r = (int)(i / nb), k = (int)(i % nb);
    const float* src = partial + (int64_t)r * nchunk * nb + k;
    float s = 0.f;
    for (int c = 0; c < nchunk; c++) s += src[(int64_t)c * nb];
    power[i] = s * scale;
}

// PCal fold: thread-private accumulators in shared memory, [bin][thread].
// TaskCoreIPP::doMaths folds the overlapped FFT windows whose running FFT
// count is a multiple of the overlap factor (TaskCoreIPP.cpp:414-418).  The
// count starts at 0 once per call (:358), runs on across the spectra of the
// call and advances after every source's FFT (:434-435), so with ns sources
// source rs folds window j of spectrum s when (ns (s novl + j) + rs) % ov == 0:
// an arithmetic progression j0, j0 + step, ... (step = ov / gcd(ns, ov)),
// possibly empty.  Each window is folded from its own start (the rotator
// index restarts), N samples from j * hop.
CS_DEV int gcd_int(int a, int b) { while (b) { int t = a % b; a = b; b = t; } return a; }

__global__ void k_pcal_fold(const uint8_t* __restrict__ planes, int64_t bytes_per_sub, int nspec, int64_t samp_per_spec,
                            int N, int ov, int novl, int ns, int rs, int T, int L, const float2* __restrict__ rot,
                            float l0, float l1, float l2, float l3, const uint32_t* __restrict__ vmask,
                            float2* __restrict__ partial, int nblk_per_row)
{
    extern __shared__ float2 pacc[];                 // [T][blockDim]
    const int row = blockIdx.y, sub = row / nspec, spec = row % nspec;
    const int nt = blockDim.x, tid = threadIdx.x;
    for (int b = 0; b < T; b++) pacc[b * nt + tid] = make_float2(0.f, 0.f);
    const uint32_t* plane = reinterpret_cast<const uint32_t*>(planes + (int64_t)sub * bytes_per_sub);
    const int step = ov / gcd_int(ns, ov);
    int j0 = -1;
    for (int j = 0; j < step && j < novl; j++)
        if (((int64_t)ns * ((int64_t)spec * novl + j) + rs) % ov == 0) { j0 = j; break; }
    const int cnt = j0 >= 0 ? (novl - 1 - j0) / step + 1 : 0;
    const int hop = N / ov, wpw = N / 16;            // 32-bit words per window
    const int64_t nwords = (int64_t)cnt * wpw;
    const float lut[4] = {l0, l1, l2, l3};
    // Sample j of word wi of a window has rotator index (16 wi + j) mod L and
    // bin that mod T.  A thread keeps the 16 rotator values and bins of its
    // current wi in registers and sums each j over the windows in a register,
    // adding the sums into its shared-memory slots when wi changes (for
    // N = 65536, whose windows have 4096 words like the 32 x 128 threads of
    // a row, never: each thread owns one wi).
    float2 acc[16], rj[16];
    int bj[16];
    int cur = -1;
    auto flush = [&]() {
#pragma unroll
        for (int j = 0; j < 16; j++) {
            if (cur >= 0) {
                float2& slot = pacc[bj[j] * nt + tid];
                slot.x += acc[j].x;
                slot.y += acc[j].y;
            }
            acc[j] = make_float2(0.f, 0.f);
        }
    };
    flush();
    for (int64_t w = (int64_t)blockIdx.x * nt + tid; w < nwords; w += (int64_t)nblk_per_row * nt) {
        const int win = (int)(w / wpw), wi = (int)(w - (int64_t)win * wpw);
        if (wi != cur) {
            flush();
            cur = wi;
            int li = (wi * 16) % L, bi = li % T;
#pragma unroll
            for (int j = 0; j < 16; j++) {
                rj[j] = __ldg(rot + li);
                bj[j] = bi;
                li++;
                bi++;
                if (li == L) li = 0, bi = 0;
                else if (bi == T) bi = 0;
            }
        }
        const int64_t wg = ((int64_t)spec * samp_per_spec + (int64_t)(j0 + win * step) * hop) / 16 + wi;
        const uint32_t word = __ldg(plane + wg);
        const uint32_t valid = vmask ? __ldg(vmask + (wg >> 1)) >> ((wg & 1) * 16) : 0xffffu;
#pragma unroll
        for (int j = 0; j < 16; j++) {
            const float x = (valid >> j) & 1u ? lut_pick4(lut, (word >> (2 * j)) & 3u) : 0.f;
            acc[j].x += x * rj[j].x;
            acc[j].y += x * rj[j].y;
        }
    }
    flush();
    __syncthreads();
    for (int b = tid; b < T; b += nt) {
        float2 s = make_float2(0.f, 0.f);
        for (int u = 0; u < nt; u++) {
            float2 v = pacc[b * nt + u];
            s.x += v.x;
            s.y += v.y;
        }
        partial[((int64_t)row * nblk_per_row + blockIdx.x) * T + b] = s;
    }
}

__global__ void k_pcal_reduce(const float2* __restrict__ partial, int rows, int nblk, int T, int ntones,
                              float2* __restrict__ bins, float2* __restrict__ tones)
{
    int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= rows) return;
    for (int b = 0; b < T; b++) {
        float2 s = make_float2(0.f, 0.f);
        for (int u = 0; u < nblk; u++) {
            float2 v = partial[((int64_t)row * nblk + u) * T + b];
            s.x += v.x;
            s.y += v.y;
        }
        bins[(int64_t)row * T + b] = s;
    }
    if (!tones) return;
    for (int k = 0; k < ntones; k++) {
        double re = 0, im = 0;
        for (int n = 0; n < T; n++) {
            float2 bv = bins[(int64_t)row * T + n];
            double sn, cs;
            sincospi(-2.0 * (double)(((int64_t)k * n) % T) / (double)T, &sn, &cs);
            re += bv.x * cs - bv.y * sn;
            im += bv.x * sn + bv.y * cs;
        }
        tones[(int64_t)row * ntones + k] = make_float2((float)(re / T), (float)(im / T));
    }
}

constexpr int PCAL_THREADS = 128;
constexpr int PCAL_BLOCKS = 32;

// CELLSPE_SPEC_CTA_FFT=1 selects the shared-memory radix-16 kernel for N =
// 32768 and 65536 instead of choosing between it and the warp four-step.
bool spec_cta_fft()
{
    static const bool v = [] {
        const char* e = getenv("CELLSPE_SPEC_CTA_FFT");
        return e && e[0] == '1';
    }();
    return v;
}

int spec_chunk(const CsSpecArgs& a) { return a.ffts_per_chunk > 0 ? a.ffts_per_chunk : SPEC_CH; }

template <int MC, int P>
int launch_power(const CsSpecArgs& a, int nchunk, cudaStream_t st)
{
    using C = SCfg<MC>;
    constexpr int M = MC * P, N = 2 * M;
    const float2* tw = a.tw_table ? a.tw_table : cs_twiddles(N);
    const float* win = a.win_table ? a.win_table : window_table(a.window, N);
    if (!tw || !win) return CS_ERR_ARG;
    size_t smem = (size_t)C::GROUPS * fpad_size(MC) * sizeof(float2) + (size_t)C::GROUPS * (M / P + 1) * sizeof(float);
    auto kern = k_spec_power<MC, P>;
    CS_CUDA_TRY(cs_smem_at_least(reinterpret_cast<const void*>(kern), (int)smem));
    dim3 grid(nchunk, a.nsub * a.nspec, P);
    kern<<<grid, C::NT, smem, st>>>(a, tw, win, nchunk, spec_chunk(a)), cs_count_launches(1);
    return (int)cudaGetLastError();
}

template <int P>
int launch_power_w(const CsSpecArgs& a, int nchunk, cudaStream_t st)
{
    constexpr int N = 2 * SW_MC * P;
    const float2* tw = a.tw_table ? a.tw_table : cs_twiddles(N);
    const float* win = a.win_table ? a.win_table : window_table(a.window, N);
    if (!tw || !win) return CS_ERR_ARG;
    if ((N / a.overlap) % 64) return launch_power<SW_MC, P>(a, nchunk, st);   // FFT starts not 16-byte aligned
    const size_t smem = (size_t)16 * SW_ROWP * sizeof(float2) + (size_t)SW_SLOTS * SW_NT * sizeof(float) + N / 16 * 4;
    auto kern = a.valid_mask ? k_spec_power_w<P, true> : k_spec_power_w<P, false>;
    CS_CUDA_TRY(cs_smem_at_least(reinterpret_cast<const void*>(kern), (int)smem));
    dim3 grid(nchunk, a.nsub * a.nspec, P);
    kern<<<grid, SW_NT, smem, st>>>(a, tw, win, nchunk, spec_chunk(a)), cs_count_launches(1);
    return (int)cudaGetLastError();
}

// N = 32768 / 65536: the warp four-step or the CTA radix-16 power kernel,
// chosen per (device, N, overlap) by timing both once on the caller's own job
// (both compute the same partial sums, so each runs once warm and once timed
// and the chosen one runs for the result); outside stream capture and where
// the calling thread allows timing (not inside service workers).  Until a
// timed choice exists, and with CELLSPE_SPEC_CTA_FFT=1, fixed choices.
std::mutex g_sp_tune_mu;
std::map<std::tuple<int, int, int>, int> g_sp_choice;   // (device, N, overlap) -> 0 warp, 1 CTA

template <int P>
int launch_power_long(const CsSpecArgs& a, int nchunk, cudaStream_t st)
{
    if (spec_cta_fft()) return launch_power<SW_MC, P>(a, nchunk, st);
    int dev = 0;
    cudaGetDevice(&dev);
    const auto key = std::make_tuple(dev, a.N, a.overlap);
    int choice = -1;
    {
        std::lock_guard<std::mutex> lk(g_sp_tune_mu);
        auto it = g_sp_choice.find(key);
        if (it != g_sp_choice.end()) choice = it->second;
    }
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    const bool can_time = cs_fstage_timing_allowed() && cudaStreamIsCapturing(st, &cap) == cudaSuccess &&
                          cap == cudaStreamCaptureStatusNone;
    if (choice < 0 && can_time) {
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        float t[2] = {1e30f, 1e30f};
        if (cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess) {
            for (int v = 0; v < 2; v++) {
                auto run = [&] { return v ? launch_power<SW_MC, P>(a, nchunk, st) : launch_power_w<P>(a, nchunk, st); };
                if (run() != 0) continue;
                cudaEventRecord(e0, st);
                const int rc = run();
                cudaEventRecord(e1, st);
                if (rc == 0 && cudaEventSynchronize(e1) == cudaSuccess) cudaEventElapsedTime(&t[v], e0, e1);
            }
        }
        cudaGetLastError();
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        choice = t[1] < 0.98f * t[0] ? 1 : 0;
        std::lock_guard<std::mutex> lk(g_sp_tune_mu);
        g_sp_choice[key] = choice;
    }
    return choice == 1 ? launch_power<SW_MC, P>(a, nchunk, st) : launch_power_w<P>(a, nchunk, st);
}

int spec_nchunk(const CsSpecArgs& a)
{
    int novl = a.overlap * a.ffts_per_spectrum - (a.overlap - 1);
    return (novl + spec_chunk(a) - 1) / spec_chunk(a);
}
}  // namespace

const float* cs_window_table(int type, int n) { return window_table(type, n); }

// Scratch layout: chunk partial spectra, then (256-byte aligned: N/2+1 is
// odd, and the phase-cal partials are float2) the phase-cal partials.
int64_t power_partial_floats(const CsSpecArgs& a)
{
    const int64_t power = (int64_t)a.nsub * a.nspec * spec_nchunk(a) * (a.N / 2 + 1);
    return (power + 63) / 64 * 64;
}

int64_t cs_spectrometer_pcal_floats(const CsSpecArgs& a)
{
    return a.tonebins > 0 ? (int64_t)a.nsub * a.nspec * PCAL_BLOCKS * a.tonebins * 2 : 0;
}

int64_t cs_spectrometer_scratch_floats(const CsSpecArgs& a)
{
    return power_partial_floats(a) + cs_spectrometer_pcal_floats(a);
}

int cs_spectrometer(const CsSpecArgs& a, cudaStream_t st)
{
    if (!a.planes || (!a.power && !a.skip_power) || !a.partial || a.nsub <= 0 || a.nspec <= 0 ||
        a.ffts_per_spectrum <= 0)
        return CS_ERR_ARG;
    if (a.overlap < 1 || a.N % (16 * a.overlap) != 0) return CS_ERR_ARG;
    if ((uintptr_t)a.planes % 16 || a.bytes_per_sub % 16) return CS_ERR_ARG;
    // every sample the spectra read must lie inside the subband plane
    if ((int64_t)a.nspec * a.ffts_per_spectrum * a.N > a.bytes_per_sub * 4) return CS_ERR_ARG;
    if (a.nsub * a.nspec > 65535) return CS_ERR_ARG;
    const int nchunk = spec_nchunk(a);
    int rc = 0;
    if (!a.skip_power) switch (a.N) {
        case 1024: rc = launch_power<512, 1>(a, nchunk, st); break;
        case 2048: rc = launch_power<1024, 1>(a, nchunk, st); break;
        case 4096: rc = launch_power<2048, 1>(a, nchunk, st); break;
        case 8192: rc = launch_power<4096, 1>(a, nchunk, st); break;
        case 16384: rc = launch_power<8192, 1>(a, nchunk, st); break;
        case 32768: rc = launch_power_long<1>(a, nchunk, st); break;
        case 65536: rc = launch_power_long<2>(a, nchunk, st); break;
        default: return CS_ERR_UNSUPPORTED;
    }
    if (rc) return rc;
    const int rows = a.nsub * a.nspec, nb = a.N / 2 + 1;
    const int novl = a.overlap * a.ffts_per_spectrum - (a.overlap - 1);
    if (!a.skip_power) {
        const float scale = (float)(1.0 / (double)novl);
        int64_t tot = (int64_t)rows * nb;
        k_spec_reduce<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(a.partial, a.power, rows, nchunk, nb, scale),
            cs_count_launches(1);
        CS_CUDA_TRY(cudaGetLastError());
    }

    if (a.tonebins > 0) {
        const int T = a.tonebins, L = a.rotatorlen;
        if (L <= 0 || L % T != 0 || a.N % L != 0 || T > 128 || !a.pcal_bins) return CS_ERR_ARG;
        const float2* rot = a.rot_table ? a.rot_table : rotator_table(L, a.pcal_offset_hz, a.fs_hz);
        if (!rot) return CS_ERR_ARG;
        float2* pp = reinterpret_cast<float2*>(a.partial + power_partial_floats(a));
        int64_t samp_per_spec = (int64_t)a.ffts_per_spectrum * a.N;
        int nt = PCAL_THREADS;
        size_t smem = (size_t)T * nt * sizeof(float2);
        CS_CUDA_TRY(cs_smem_at_least(reinterpret_cast<const void*>(k_pcal_fold), (int)smem));
        const int ns = a.pcal_sources > 0 ? a.pcal_sources : 1;
        k_pcal_fold<<<dim3(PCAL_BLOCKS, rows), nt, smem, st>>>(a.planes, a.bytes_per_sub, a.nspec, samp_per_spec, a.N,
                                                               a.overlap, novl, ns, a.pcal_source, T, L, rot, a.lut[0],
                                                               a.lut[1], a.lut[2], a.lut[3], a.valid_mask, pp,
                                                               PCAL_BLOCKS), cs_count_launches(1);
        CS_CUDA_TRY(cudaGetLastError());
        k_pcal_reduce<<<(rows + 63) / 64, 64, 0, st>>>(pp, rows, PCAL_BLOCKS, T, a.ntones, a.pcal_bins, a.pcal_tones), cs_count_launches(1);
        CS_CUDA_TRY(cudaGetLastError());
    }
    return 0;
}
