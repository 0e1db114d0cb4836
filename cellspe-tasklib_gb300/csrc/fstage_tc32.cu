// K-b/K-c on the tensor cores, 32-segment units: the FX F stage for N = 2048
// with FP16 spectra written k-blocked (128-byte runs of 32 Re then 32 Im
// halves per channel, input and 32-segment block, which the tcgen05 X stage
// reads), for K and kp multiples of 32: the lockstep form in layout 1
// (__half [C][S_out][kp/32][2][32]), the warp-specialised form in the
// channel-grouped layout 2 ([C/16][S_out][kp/32][16] runs; cs_fstage_layout).
//
// The real 2048-point DFT X[c] = sum_n x[n] W_2048^(n c), c < 1024, as a
// four-step transform with both passes on the tensor cores (FP16 operands,
// FP32 accumulators in TMEM).  With n = n2 + 32 n1 (n1 < 64, n2 < 32) and
// c = k1 + 64 k2:
//     Y[k1][n2] = sum_n1 x[n2 + 32 n1] W_64^(n1 k1)        pass 1
//     Z[k1][n2] = Y[k1][n2] W_2048^(n2 k1)                 CUDA cores
//     X[k1 + 64 k2] = sum_n2 Z[k1][n2] W_32^(n2 k2)        pass 2
// The input is real, so X[2048 - c] = conj(X[c]) and only k1 = 0..32 is
// needed: pass 2 runs for k1 < 32 over all 32 k2 and gives the channels with
// c mod 64 < 32 directly (k2 < 16) and those with c mod 64 > 32 as conj(X) of
// the mirror bin (k2 >= 16); the 16 channels with c mod 64 = 32 come from the
// k1 = 32 row (real Y) through one more pass-2 product per unit.  Per segment
// the CUDA cores twiddle 1024 values instead of 2048.
//
// Work unit = 32 consecutive segments of one input, in 8 quads of 4
// segments.  Per quad:
//  * decode: 2-bit samples -> B1 (FP16, MN-major: K = n1, N = (segment, n2))
//  * pass 1: D1 = A1 B1, A1 the constant DFT-64 rows (TMEM lane quarter q
//    holds Re rows 32q..32q+7 and Im rows 32q+8..32q+15 of k1 = 8q..8q+7, and
//    quarter 0 the k1 = 32 row in lanes 16..23), 128 x 128 x 64
//  * epilogue 1: Z = Y W -> A2 (FP16, K-major rows (segment, k1), K = Re | Im
//    of n2); the k1 = 32 values -> A2' (row = segment of the unit)
//  * pass 2: D2 = A2 B2, B2 the constant DFT-32 as a real 64 x 64 operand
//  * epilogue 2: delay / fringe phasor, channel scale, FP16 -> staging
//    [segment][channel] (Re, Im) words
// and per unit pass 2' (D2' = A2' B2) and its epilogue for the k1 = 32
// channels, then the write-out: each (channel, input, 32-segment block) is one
// 128-byte run (32 Re halves, 32 Im halves), written by the workers from the
// staging with 16-byte stores, 4 lanes per 64-byte half-run.
//
// Warps 0..15 are the workers (decode, both epilogues, write-out); warp 16
// owns TMEM and one of its threads issues the MMAs.  The workers' loop is skewed so
// that they never wait on an MMA they just enabled: iteration j runs
// epilogue 1 of quad j, the decode of quad j+1 and epilogue 2 of quad j-1, so
// pass 2 of quad j runs during the decode and epilogue 2, and pass 1 of quad
// j+1 during epilogue 2 (A2 and D2 double-buffered, D1 double-buffered in
// TMEM).  Every mbarrier wait is bounded
// (~2 s): on timeout the threads record an error code, leave their loops
// together (worker votes), drain the tensor pipe and free TMEM.  One worker
// thread polls each barrier the workers wait on and the vote that follows
// releases the others (no spinning warps); the workers arrive once per warp.
#include "common.cuh"
#include "kernels.h"
#include "tcgen05.cuh"

#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <vector>

namespace {

constexpr int FN = 2048, FC = 1024;
constexpr int QS = 4;                                 // segments per quad
constexpr int US = 32;                                // segments per unit
constexpr int QUADS = US / QS;
constexpr int WORKERS = 512, THREADS = WORKERS + 32;  // + the MMA warp
constexpr int MMA_WARP = WORKERS / 32;
constexpr int RAWC = 34;                              // 16-byte raw chunks per segment (2048 samples + slack)
// constant operands (pre-swizzled on the host)
constexpr int OFF_A1 = 0;                             // DFT-64: 128 rows x 128 B, K-major, 128-byte swizzle
constexpr int OFF_B2 = 16384;                         // DFT-32: 64 rows x 128 B
constexpr int CONST_BYTES = 24576;
constexpr int OFF_B1 = CONST_BYTES;                   // samples of one quad: 2 atoms x (64 rows x 128 B)
constexpr int B1_BYTES = 16384;
constexpr int OFF_A2 = OFF_B1 + B1_BYTES;             // Z of a quad: 2 buffers x 128 rows x 128 B
constexpr int A2_BYTES = 16384;
// Z of the k1 = 32 row, row = segment of the unit: 2 regions of 32 rows
// (units alternate).  Pass 2' reads a 128-row window from a region's start;
// window rows 32..127 fall on the other region and the staging, and only
// feed TMEM lanes 32..127 of D2', which are never read.
constexpr int OFF_A2P = OFF_A2 + 2 * A2_BYTES;
constexpr int A2P_REGION = 32 * 128;
constexpr int STG_PITCH = FC + 1;                     // words per staging row (one row per segment)
constexpr int OFF_STG = OFF_A2P + 2 * A2P_REGION;     // staging: [US][STG_PITCH] half2 (Re, Im)
constexpr int STG_BYTES = US * STG_PITCH * 4;
constexpr int OFF_RAW = OFF_STG + STG_BYTES;          // 2 x QS x RAWC x 16
constexpr int RAW_BYTES = QS * RAWC * 16;
constexpr int OFF_OFFS = OFF_RAW + 2 * RAW_BYTES;     // sample offsets: 2 x QS ints
constexpr int OFF_LUT = OFF_OFFS + 2 * QS * 4;        // 16 half2 pair levels
constexpr int OFF_BAR = OFF_LUT + 64;                 // mbarriers
constexpr int NBAR = 12;
constexpr int OFF_SLOT = OFF_BAR + 8 * NBAR;
constexpr int SMEM_USED = OFF_SLOT + 16;
constexpr int SMEM_BYTES = SMEM_USED + 1024;          // + alignment of the base to 1024 B
constexpr uint32_t TMEM_COLS = 512;                   // D1: 0, 128; D2: 256, 320; D2': 384
constexpr uint32_t COL_D1 = 0, COL_D2 = 256, COL_D2P = 384;
constexpr long long WAIT_CYCLES = 4000000000LL;       // ~2 s

// barriers
constexpr int B_B1FULL = 0, B_D1FULL = 1, B_EPI1 = 2, B_D2FULL0 = 3, B_EPI2_0 = 5, B_D2PFULL = 7, B_EPI2P = 8,
              B_DRAIN = 9;
// error codes
constexpr unsigned E_MMA_WAIT = 1, E_WORKER_WAIT = 2;

__device__ unsigned g_fst32_error;

static_assert(SMEM_BYTES <= 227 * 1024, "shared memory");
static_assert(OFF_B1 % 1024 == 0 && OFF_A2 % 1024 == 0 && OFF_A2P % 1024 == 0 && A2P_REGION % 1024 == 0,
              "swizzle atoms need 1024-B alignment");
static_assert(OFF_A2P + A2P_REGION + 16384 <= OFF_STG + US * STG_PITCH * 4, "pass-2' windows inside shared memory");

CS_DEV void cp_async16(uint32_t dst, const void* src, bool valid)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(valid ? 16 : 0)
                 : "memory");
}
CS_DEV void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
CS_DEV void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

static_assert(WORKERS == 512, "the named barriers below count 512 workers");
CS_DEV void worker_bar() { asm volatile("bar.sync 1, 512;" ::: "memory"); }
// all workers agree on `ok` (and synchronise)
CS_DEV bool worker_vote(bool ok)
{
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "bar.red.and.pred q, 1, 512, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(r)
        : "r"(ok ? 1u : 0u)
        : "memory");
    return r != 0;
}

// Worker arrival on a barrier that counts warps: every lane's earlier writes
// (and its own fences) are ordered before lane 0's arrive by the warp sync.
CS_DEV void warp_arrive(uint32_t bar)
{
    __syncwarp();
    if ((threadIdx.x & 31) == 0) tc::mbar_arrive(bar);
}

// After tcgen05.wait::ld: ties the loaded registers to that point.
CS_DEV void pin16(uint32_t (&r)[16])
{
#pragma unroll
    for (int i = 0; i < 16; i++) asm volatile("" : "+r"(r[i]));
}

// byte offset of element (row, k) of a 128-byte-swizzled K-major operand
// (rows of 64 FP16, 8-row groups every 1024 B)
CS_DEV uint32_t sw128(uint32_t row, uint32_t k)
{
    return row * 128 + ((((k >> 3) ^ row) & 7) << 4) + (k & 7) * 2;
}

CS_DEV uint32_t h2u(__half2 v) { return *reinterpret_cast<const uint32_t*>(&v); }

struct Tc32Args {
    CsFStageArgs f;
    const uint4* consts;      // A1 + B2, CONST_BYTES, already swizzled
    int units_k;              // 32-segment units per input = K / 32
    int64_t units;            // S * units_k
    int nkb;                  // kp / 32: 32-segment blocks per output row
    int s_rows;               // S_out
};

template <bool PHASE, bool SCALE>
__global__ void __launch_bounds__(THREADS, 1) k_fx_fstage_tc32(const __grid_constant__ Tc32Args args)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    // offset from the shared array itself (not an integer round trip), so that
    // the compiler keeps shared-space 32-bit addressing for every access
    unsigned char* sm = smem_raw + ((1024u - (tc::smem_u32(smem_raw) & 1023u)) & 1023u);
    const uint32_t sbase = tc::smem_u32(sm);
    const CsFStageArgs& a = args.f;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tid = threadIdx.x;
    const uint32_t bar0 = sbase + OFF_BAR;
    auto bar = [&](int i) { return bar0 + 8u * (uint32_t)i; };
    uint32_t* slot = reinterpret_cast<uint32_t*>(sm + OFF_SLOT);
    int* offs = reinterpret_cast<int*>(sm + OFF_OFFS);
    __half2* lut2 = reinterpret_cast<__half2*>(sm + OFF_LUT);

    // constants into shared memory, A2' zeroed (its rows past the unit's 32
    // segments are read by the MMA but never used), barriers, TMEM
    for (int i = tid; i < CONST_BYTES / 16; i += THREADS)
        reinterpret_cast<uint4*>(sm)[i] = __ldg(args.consts + i);
    for (int i = tid; i < 2 * A2P_REGION / 16; i += THREADS)
        reinterpret_cast<uint4*>(sm + OFF_A2P)[i] = make_uint4(0, 0, 0, 0);
    if (tid < 16) {
        // the level table is in parameter space: read with constant indices only
        const float l0 = a.lut[0], l1 = a.lut[1], l2 = a.lut[2], l3 = a.lut[3];
        auto lv = [&](int c) { return c == 0 ? l0 : c == 1 ? l1 : c == 2 ? l2 : l3; };
        lut2[tid] = __floats2half2_rn(lv(tid & 3), lv(tid >> 2));
    }
    if (tid == 0) {
        tc::mbar_init(bar(B_B1FULL), WORKERS / 32);
        tc::mbar_init(bar(B_D1FULL), 1);
        tc::mbar_init(bar(B_EPI1), WORKERS / 32);
        tc::mbar_init(bar(B_D2FULL0), 1);
        tc::mbar_init(bar(B_D2FULL0 + 1), 1);
        tc::mbar_init(bar(B_EPI2_0), WORKERS / 32);
        tc::mbar_init(bar(B_EPI2_0 + 1), WORKERS / 32);
        tc::mbar_init(bar(B_D2PFULL), 1);
        tc::mbar_init(bar(B_EPI2P), WORKERS / 32);
        tc::mbar_init(bar(B_DRAIN), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == MMA_WARP) tc::tmem_alloc(tc::smem_u32(slot), TMEM_COLS);
    tc::fence_proxy_async();                       // constant operands -> tensor core
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = *slot;

    const int64_t units = args.units;
    const int nunits = (blockIdx.x < units) ? (int)((units - 1 - blockIdx.x) / gridDim.x + 1) : 0;
    const int nquads = nunits * QUADS;
    const int K = a.K;

    if (warp == MMA_WARP) {
        // ------------------------------ MMA issuer ------------------------------
        if (lane == 0) {
            const uint32_t id1 = tc::idesc_f16(128, 128, false, false, true);    // B1 MN-major
            const uint32_t id2 = tc::idesc_f16(128, 64, false, false, false);
            bool ok = true;
            for (int j = 0; j < nquads && ok; j++) {
                const int b = j & 1;
                // B1 holds quad j (decoded after epilogue 1 of quad j-1, which
                // freed D1 buffer b of quad j-2)
                ok = tc::mbar_wait(bar(B_B1FULL), (uint32_t)j & 1, &g_fst32_error, E_MMA_WAIT, WAIT_CYCLES);
                if (!ok) break;
                tc::fence_after();
                const uint32_t b1 = sbase + OFF_B1;
#pragma unroll
                for (int kk = 0; kk < 4; kk++) {
                    const uint64_t da = tc::smem_desc(sbase + OFF_A1 + 32u * kk, 16, 1024, tc::SW128);
                    // MN-major: 8-row K groups every 1024 B, 64-wide N atoms every 8192 B
                    const uint64_t db = tc::smem_desc(b1 + 2048u * kk, 8192, 1024, tc::SW128);
                    tc::mma_f16(tmem + COL_D1 + 128u * b, da, db, id1, kk ? 1u : 0u);
                }
                tc::commit(bar(B_D1FULL));
                // A2 buffer b (and the quad's A2' rows) written by epilogue 1 of quad j
                ok = tc::mbar_wait(bar(B_EPI1), (uint32_t)j & 1, &g_fst32_error, E_MMA_WAIT, WAIT_CYCLES);
                // D2 buffer b free: epilogue 2 of quad j-2 done
                if (ok && j >= 2)
                    ok = tc::mbar_wait(bar(B_EPI2_0 + b), (uint32_t)((j - 2) >> 1) & 1, &g_fst32_error, E_MMA_WAIT,
                                       WAIT_CYCLES);
                if (!ok) break;
                tc::fence_after();
#pragma unroll
                for (int kk = 0; kk < 4; kk++) {
                    const uint64_t da = tc::smem_desc(sbase + OFF_A2 + (uint32_t)b * A2_BYTES + 32u * kk, 16, 1024, tc::SW128);
                    const uint64_t db = tc::smem_desc(sbase + OFF_B2 + 32u * kk, 16, 1024, tc::SW128);
                    tc::mma_f16(tmem + COL_D2 + 64u * b, da, db, id2, kk ? 1u : 0u);
                }
                tc::commit(bar(B_D2FULL0 + b));
                if (j % QUADS == QUADS - 1) {
                    // the unit's k1 = 32 rows are complete; D2' free once the
                    // previous unit's epilogue 2' is done
                    const int u = j / QUADS;
                    if (u >= 1)
                        ok = tc::mbar_wait(bar(B_EPI2P), (uint32_t)(u - 1) & 1, &g_fst32_error, E_MMA_WAIT,
                                           WAIT_CYCLES);
                    if (!ok) break;
                    tc::fence_after();
#pragma unroll
                    for (int kk = 0; kk < 4; kk++) {
                        const uint64_t da = tc::smem_desc(sbase + OFF_A2P + (uint32_t)(u & 1) * A2P_REGION + 32u * kk,
                                                          16, 1024, tc::SW128);
                        const uint64_t db = tc::smem_desc(sbase + OFF_B2 + 32u * kk, 16, 1024, tc::SW128);
                        tc::mma_f16(tmem + COL_D2P, da, db, id2, kk ? 1u : 0u);
                    }
                    tc::commit(bar(B_D2PFULL));
                }
            }
            // completes once every MMA issued above has finished
            tc::commit(bar(B_DRAIN));
            tc::mbar_wait(bar(B_DRAIN), 0, &g_fst32_error, E_MMA_WAIT, WAIT_CYCLES);
        }
        __syncwarp();
    } else {
        // ------------------------------ workers ------------------------------
        const int q = warp & 3, h = warp >> 2;        // TMEM lane quarter, quarter of the work
        const int64_t chunks = a.bytes_per_input >> 4;
        const int k1 = 8 * q + (lane >> 2);           // epilogue 1: this thread's k1 (< 32)

        // epilogue-1 twiddles W_2048^(n2 k1), n2 = 8 m + 2 (lane % 4) + e
        float2 tw[4][2];
#pragma unroll
        for (int m = 0; m < 4; m++)
#pragma unroll
            for (int e = 0; e < 2; e++) {
                const int n2 = 8 * m + 2 * (lane & 3) + e;
                float sn, cs;
                sincospif(-(float)((n2 * k1) & 2047) / 1024.0f, &sn, &cs);
                tw[m][e] = make_float2(cs, sn);
            }
        // epilogue 1 stores: A2 row 32 h + k1 (fixed per thread), K positions
        // 8 m + 2 (lane % 4) (Re) and 32 + that (Im).  Their swizzled byte
        // offsets are sw128(row, 0) + 4 (lane % 4) with the 16-byte chunk index
        // XORed by m (and by 4 more for Im): e1base ^ (m << 4) ^ (e << 6)
        const uint32_t e1base = sw128(32 * h + k1, 2 * (lane & 3));
        // the k1 = 32 row (quarter 0): this thread's (m, e) and W_64^(n2)
        const int m32 = (lane >> 2) & 3, e32 = lane >> 4;
        const int n2_32 = 8 * m32 + 2 * (lane & 3) + e32;
        float2 tw32;
        {
            float sn, cs;
            sincospif(-(float)n2_32 / 32.0f, &sn, &cs);
            tw32 = make_float2(cs, sn);
        }

        // unit u of this CTA -> (input, 32-segment block); 32-bit arithmetic
        // (a 64-bit division is a long FP64-assisted sequence on the GPU)
        auto unit_of = [&](int u, int& s, int& kb) {
            const uint32_t uu = blockIdx.x + (uint32_t)u * gridDim.x;
            const uint32_t si = uu / (uint32_t)args.units_k;
            s = (int)si;
            kb = (int)(uu - si * (uint32_t)args.units_k);
        };
        // raw chunks of quad j -> raw buffer j & 1 (zero outside the input)
        auto fetch = [&](int j) {
            int s, kb;
            unit_of(j / QUADS, s, kb);
            const int kq = kb * US + (j % QUADS) * QS;
            const unsigned char* base = a.raw + (int64_t)s * a.bytes_per_input;
            const uint32_t dst0 = sbase + OFF_RAW + (uint32_t)(j & 1) * RAW_BYTES;
            for (int i = tid; i < QS * RAWC; i += WORKERS) {
                const int g = i / RAWC, c = i % RAWC, k = kq + g;
                const int64_t start = a.start_sample + (int64_t)k * FN + (a.shift ? __ldg(a.shift + (int64_t)s * K + k) : 0);
                const int64_t ci = (start >> 6) + c;
                const bool ok = ci >= 0 && ci < chunks;
                cp_async16(dst0 + 16u * i, ok ? base + 16 * ci : a.raw, ok);
                if (c == 0) offs[(j & 1) * QS + g] = (int)(start & 63);
            }
            cp_async_commit();
        };
        // unpack quad j (raw buffer j & 1) -> B1:
        // element (n1, 32 g + n2) = sample 32 n1 + n2 of segment g
        auto decode = [&](int j) {
            const uint32_t* rw0 = reinterpret_cast<const uint32_t*>(sm + OFF_RAW + (j & 1) * RAW_BYTES);
            unsigned char* b1 = sm + OFF_B1;
            {
                const int idx = tid;                      // QS x 128 words, one per worker
                const int g = idx >> 7, wd = idx & 127;
                const int off = offs[(j & 1) * QS + g];
                const uint32_t* rw = rw0 + g * RAWC * 4 + (off >> 4) + wd;
                const uint32_t bits = __funnelshift_r(rw[0], rw[1], 2 * (off & 15));
                uint32_t hv[8];
#pragma unroll
                for (int p = 0; p < 8; p++) hv[p] = h2u(lut2[(bits >> (4 * p)) & 15u]);
                const int n1 = wd >> 1;
                const int chunk = 4 * (g & 1) + 2 * (wd & 1);
                unsigned char* rowp = b1 + (g >> 1) * 8192 + n1 * 128;
                *reinterpret_cast<uint4*>(rowp + (((chunk ^ n1) & 7) << 4)) = make_uint4(hv[0], hv[1], hv[2], hv[3]);
                *reinterpret_cast<uint4*>(rowp + ((((chunk + 1) ^ n1) & 7) << 4)) = make_uint4(hv[4], hv[5], hv[6], hv[7]);
            }
        };
        uint32_t* stg = reinterpret_cast<uint32_t*>(sm + OFF_STG);
        // (B, D) = exp(i (phase0 + cstart dphase)), exp(i cstep dphase) of segment k
        // of input s: the delay model's phasor at the first channel a thread
        // writes and its step to the next (the identity without a delay model)
#define TC32_PHASOR(s_, k_, cstart, cstep)                                              \
        float2 B = make_float2(1.f, 0.f), D = B;                                        \
        if (PHASE) {                                                                    \
            const int64_t sk = (int64_t)(s_) * K + (k_);                                \
            const float ph0 = __ldg(a.phase0 + sk), dph = __ldg(a.dphase + sk);         \
            float sn, cs;                                                               \
            sincosf(ph0 + (cstart) * dph, &sn, &cs);                                    \
            B = make_float2(cs, sn);                                                    \
            sincosf((cstep) * dph, &sn, &cs);                                           \
            D = make_float2(cs, sn);                                                    \
        }
        // one spectrum value X of channel c_ (unit-relative segment seg_) into the staging
#define TC32_STAGE(seg_, s_, c_, X_)                                                    \
        {                                                                               \
            float2 X = (X_);                                                            \
            if (PHASE) {                                                                \
                X = cmul(X, B);                                                         \
                B = cmul(B, D);                                                         \
            }                                                                           \
            if (SCALE) X = cscale(X, __ldg(scl + (c_)));                                \
            stg[(seg_) * STG_PITCH + (c_)] = h2u(__floats2half2_rn(X.x, X.y));          \
        }

        bool ok = true;
        if (nquads > 0) {
            fetch(0);
            if (nquads > 1) fetch(1);
            cp_async_wait_all();
            worker_bar();
            decode(0);
            tc::fence_proxy_async();
            warp_arrive(bar(B_B1FULL));
        }
        // Iteration j: one wait (worker thread 0 polls D1 of quad j, D2 of
        // quad j-1 and, at a unit's end, D2'; the vote releases the others,
        // and every thread's raw-word copies have landed before it), the TMEM
        // loads of both epilogues issued together, then epilogue 1 (j), the
        // decode of quad j+1, the fetch of quad j+2 and epilogue 2 (j-1).
        for (int j = 0; j <= nquads; j++) {
            const bool do1 = j < nquads, do2 = j >= 1;
            const int jj = j - 1;
            const bool uend = do2 && (jj % QUADS == QUADS - 1);
            cp_async_wait_all();
            ok = true;
            if (tid == 0) {
                if (do1) ok = tc::mbar_wait(bar(B_D1FULL), (uint32_t)j & 1, &g_fst32_error, E_WORKER_WAIT, WAIT_CYCLES);
                if (ok && do2)
                    ok = tc::mbar_wait(bar(B_D2FULL0 + (jj & 1)), (uint32_t)(jj >> 1) & 1, &g_fst32_error,
                                       E_WORKER_WAIT, WAIT_CYCLES);
                if (ok && uend)
                    ok = tc::mbar_wait(bar(B_D2PFULL), (uint32_t)(jj / QUADS) & 1, &g_fst32_error, E_WORKER_WAIT,
                                       WAIT_CYCLES);
            }
            if (!worker_vote(ok)) { ok = false; break; }
            tc::fence_after();
            uint32_t r[16], re[8], im[8];
            const uint32_t d1 = tmem + COL_D1 + 128u * (j & 1) + 32u * h;
            if (do1) tc::tmem_ld_16x256b_x4(d1 + ((uint32_t)(32 * q) << 16), r);
            if (do2) {
                const uint32_t d2 = tmem + COL_D2 + 64u * (jj & 1) + ((uint32_t)(32 * q) << 16);
                tc::tmem_ld_32x32b_x8(d2 + 8u * h, re);
                tc::tmem_ld_32x32b_x8(d2 + 32u + 8u * h, im);
            }
            tc::tmem_ld_wait();
            pin16(r);
#pragma unroll
            for (int i = 0; i < 8; i++) {
                asm volatile("" : "+r"(re[i]));
                asm volatile("" : "+r"(im[i]));
            }
            if (do1) {
                // ---- epilogue 1: Y -> Z = Y W_2048^(n2 k1) -> A2 buffer j & 1; warp (q, h):
                // TMEM lane quarter q (k1 = 8q..8q+7), segment h of the quad ----
                {
                    const int b = j & 1, qd = j % QUADS, u = j / QUADS, g = h;
                    unsigned char* a2 = sm + OFF_A2 + b * A2_BYTES;
#pragma unroll
                    for (int m = 0; m < 4; m++) {
                        const float2 y0 = make_float2(__uint_as_float(r[4 * m]), __uint_as_float(r[4 * m + 2]));
                        const float2 y1 = make_float2(__uint_as_float(r[4 * m + 1]), __uint_as_float(r[4 * m + 3]));
                        const float2 z0 = cmul(y0, tw[m][0]), z1 = cmul(y1, tw[m][1]);
                        *reinterpret_cast<uint32_t*>(a2 + (e1base ^ (m << 4))) = h2u(__floats2half2_rn(z0.x, z1.x));
                        *reinterpret_cast<uint32_t*>(a2 + (e1base ^ (m << 4) ^ 64u)) = h2u(__floats2half2_rn(z0.y, z1.y));
                    }
                    if (q == 0) {
                        // lanes 16..23 hold copies of the real k1 = 32 row: thread
                        // (lane) takes column 8 m32 + 2 (lane % 4) + e32 of its copy
                        // (loaded here, by the four warps of quarter 0 only, which
                        // keeps it out of the other warps' register budget)
                        uint32_t r32[16];
                        tc::tmem_ld_16x256b_x4(d1 + (16u << 16), r32);
                        tc::tmem_ld_wait();
                        pin16(r32);
                        // y = r32[4 m32 + e32] as selects on constant indices
                        // (an indexed read would put r32 in local memory)
                        const bool m1 = m32 & 1, m2 = m32 & 2;
                        const uint32_t ya = m2 ? (m1 ? r32[12] : r32[8]) : (m1 ? r32[4] : r32[0]);
                        const uint32_t yb = m2 ? (m1 ? r32[13] : r32[9]) : (m1 ? r32[5] : r32[1]);
                        const float y = __uint_as_float(e32 ? yb : ya);
                        unsigned char* a2p = sm + OFF_A2P + (u & 1) * A2P_REGION;
                        const uint32_t prow = QS * qd + g;     // segment of the unit
                        *reinterpret_cast<__half*>(a2p + sw128(prow, n2_32)) = __float2half_rn(y * tw32.x);
                        *reinterpret_cast<__half*>(a2p + sw128(prow, 32 + n2_32)) = __float2half_rn(y * tw32.y);
                    }
                }
                tc::fence_before();
                tc::fence_proxy_async();
                warp_arrive(bar(B_EPI1));
                // B1 is free (pass 1 of quad j completed) and the raw words of
                // quad j+1 are in shared memory (waited before the vote)
                if (j + 1 < nquads) {
                    decode(j + 1);
                    tc::fence_proxy_async();
                    warp_arrive(bar(B_B1FULL));
                }
                // raw buffer j & 1 was read by decode(j) before this iteration's vote
                if (j + 2 < nquads) fetch(j + 2);
            }
            if (do2) {
                const int u = jj / QUADS, b = jj & 1, qd = jj % QUADS;
                int s, kb;
                unit_of(u, s, kb);
                const float* scl = SCALE ? a.scale + (int64_t)s * FC : nullptr;
                // ---- epilogue 2: X -> phasor, scale -> FP16 staging; warp (q, h): lane
                // quarter q = segment q of the quad, lane = k1, k2 in [8 h, 8 h + 8) ----
                {
                    const int kk1 = lane;                       // k1 of this TMEM lane
                    const int seg = QS * qd + q, k = kb * US + seg;
                    if (h < 2) {
                        // c = k1 + 64 k2, k2 = 8 h + i < 16
                        const int c0 = kk1 + 512 * h;
                        TC32_PHASOR(s, k, (float)c0, 64.f)
#pragma unroll
                        for (int i = 0; i < 8; i++)
                            TC32_STAGE(seg, s, c0 + 64 * i, make_float2(__uint_as_float(re[i]), __uint_as_float(im[i])))
                    } else if (kk1 > 0) {
                        // c = 2048 - k1 - 64 k2 (k2 = 8 h + i >= 16) holds conj(X[k1 + 64 k2])
                        const int c0 = FC - kk1 - 512 * (h - 2);
                        TC32_PHASOR(s, k, (float)c0, -64.f)
#pragma unroll
                        for (int i = 0; i < 8; i++)
                            TC32_STAGE(seg, s, c0 - 64 * i, make_float2(__uint_as_float(re[i]), -__uint_as_float(im[i])))
                    }
                }
                tc::fence_before();
                warp_arrive(bar(B_EPI2_0 + b));
                if (uend) {
                    // ---- the unit's k1 = 32 channels (c = 32 + 64 k2, k2 < 16): warps
                    // 0 and 4 (lane quarter 0: lane = segment of the unit) ----
                    if (q == 0 && h < 2) {
                        uint32_t re[8], im[8];
                        tc::tmem_ld_32x32b_x8(tmem + COL_D2P + 8u * h, re);
                        tc::tmem_ld_32x32b_x8(tmem + COL_D2P + 32u + 8u * h, im);
                        tc::tmem_ld_wait();
#pragma unroll
                        for (int i = 0; i < 8; i++) {
                            asm volatile("" : "+r"(re[i]));
                            asm volatile("" : "+r"(im[i]));
                        }
                        const int seg = lane, k = kb * US + seg, c0 = 32 + 512 * h;
                        TC32_PHASOR(s, k, (float)c0, 64.f)
#pragma unroll
                        for (int i = 0; i < 8; i++)
                            TC32_STAGE(seg, s, c0 + 64 * i, make_float2(__uint_as_float(re[i]), __uint_as_float(im[i])))
                    }
                    tc::fence_before();
                    warp_arrive(bar(B_EPI2P));
                    worker_bar();                               // the unit's staging is complete
                    // ---- write-out: (channel, 8-segment group) tasks, 4 lanes per channel ----
                    __half* out = reinterpret_cast<__half*>(a.out);
                    const int64_t row0 = (int64_t)s * args.nkb + kb;       // run index of channel 0
                    const int64_t crow = (int64_t)args.s_rows * args.nkb;   // runs between channels
#pragma unroll 2
                    for (int r = 0; r < (FC * 4) / WORKERS; r++) {
                        const int task = r * WORKERS + tid;
                        const int c = task >> 2, g4 = task & 3;
                        const uint32_t* col = stg + 8 * g4 * STG_PITCH + c;
                        uint32_t w[8];
#pragma unroll
                        for (int i = 0; i < 8; i++) w[i] = col[i * STG_PITCH];
                        __half* run = out + ((int64_t)c * crow + row0) * 64 + 8 * g4;
                        *reinterpret_cast<uint4*>(run) =
                            make_uint4(__byte_perm(w[0], w[1], 0x5410), __byte_perm(w[2], w[3], 0x5410),
                                       __byte_perm(w[4], w[5], 0x5410), __byte_perm(w[6], w[7], 0x5410));
                        *reinterpret_cast<uint4*>(run + 32) =
                            make_uint4(__byte_perm(w[0], w[1], 0x7632), __byte_perm(w[2], w[3], 0x7632),
                                       __byte_perm(w[4], w[5], 0x7632), __byte_perm(w[6], w[7], 0x7632));
                    }
                    worker_bar();                               // staging free for the next unit
                }
            }
        }
#undef TC32_PHASOR
#undef TC32_STAGE
        cp_async_wait_all();
        tc::fence_before();
    }
    __syncthreads();
    if (warp == MMA_WARP) {
        tc::fence_after();
        tc::tmem_dealloc(tmem, TMEM_COLS);
    }
}

// ---------------------------------------------------------------------------
// Warp-specialised form (CELLSPE_FSTAGE_TC32=2): the same transform, but each
// phase has warps of its own and the phases hand buffers to each other
// through mbarriers, so they run concurrently instead of in step between
// CTA-wide barriers:
//   warps 0-3   epilogue 1 (TMEM lane quarter = warp), all 4 segments of a
//               quad, and each warp one segment's share of the k1 = 32 row
//   warps 4-7   epilogue 2 (lane quarter = segment of the quad) into the
//               unit's staging, whose two 16-segment halves the write-out
//               drains in turn
//   warps 8-11  decode into B1 (a byte_perm of the four levels per pair of
//               samples, no table in shared memory)
//   warps 12-15 write-out of a staging half: per channel and plane 16
//               segments, two lanes' 16 bytes making one whole sector; in
//               the channel-grouped layout a group's 16 channels of the
//               unit lie in one 2 KB stretch, so the DRAM sees long runs.
//               After a unit's second half warp 12 (lane quarter 0, lane =
//               segment) writes the unit's k1 = 32 channels from pass 2'
//               straight to the spectra.
//   warp 16     TMEM owner and MMA issuer; pass 1 of quad j + 1 is issued
//               before pass 2 of quad j, so epilogue 1 finds its next quad
//               ready
//   warp 17     raw fetch: bulk copies into NRAW buffers, up to NRAW quads
//               ahead of the decode
// A group's first thread polls the barriers (bounded waits) and a
// named-barrier vote of the group releases the others; a failed wait ends
// that group's loop, and every group's waits are bounded, so all reach the
// final barrier.
// ---------------------------------------------------------------------------
constexpr int WS_E1 = 0, WS_E2 = 4, WS_DEC = 8, WS_WO = 12, WS_MMA = 16, WS_FETCH = 17;
constexpr int WS_THREADS = 18 * 32;
// shared memory of this form: constants, B1, A2 x 2, A2' x 2, the unit's
// staging [US][WS_STG_PITCH] (pitch = 2 mod 32 words: the write-out's two
// 8-segment groups of a channel fall 16 banks apart), raw x NRAW, offsets,
// table, barriers
constexpr int NRAW = 4;                               // raw buffers
constexpr int WS_SH = US / 2;                         // segments per staging half
constexpr int WS_STG_PITCH = FC + 2;
constexpr int WS_OFF_B1 = CONST_BYTES;
constexpr int WS_OFF_A2 = WS_OFF_B1 + B1_BYTES;
constexpr int WS_OFF_A2P = WS_OFF_A2 + 2 * A2_BYTES;
constexpr int WS_OFF_STG = WS_OFF_A2P + 2 * A2P_REGION;
constexpr int WS_OFF_RAW = WS_OFF_STG + US * WS_STG_PITCH * 4;
constexpr int WS_OFF_OFFS = WS_OFF_RAW + NRAW * RAW_BYTES;
constexpr int WS_OFF_LUT = WS_OFF_OFFS + NRAW * QS * 4;
constexpr int WS_OFF_BAR = WS_OFF_LUT + 64;
constexpr int WS_NBAR = 26;
constexpr int WS_OFF_SLOT = WS_OFF_BAR + 8 * WS_NBAR;
constexpr int WS_SMEM_BYTES = WS_OFF_SLOT + 16 + 1024;   // + alignment of the base to 1024 B
// barriers ([2]: by quad parity or staging half, [NRAW]: by raw buffer)
constexpr int WB_B1FULL = 0, WB_D1FULL = 1, WB_E1DONE = 3, WB_D2FULL = 5, WB_E2DONE = 7, WB_D2PFULL = 9,
              WB_E2PDONE = 11, WB_STGFULL = 12, WB_STGFREE = 14, WB_DRAIN = 16, WB_RAWFULL = 17,
              WB_RAWFREE = WB_RAWFULL + NRAW;
static_assert(WB_RAWFREE + NRAW <= WS_NBAR, "barriers");
static_assert(WS_SMEM_BYTES <= 227 * 1024, "shared memory");
static_assert(WS_OFF_B1 % 1024 == 0 && WS_OFF_A2 % 1024 == 0 && WS_OFF_A2P % 1024 == 0,
              "swizzle atoms need 1024-B alignment");
static_assert(WS_OFF_A2P + A2P_REGION + 16384 <= WS_OFF_RAW, "pass-2' windows inside shared memory");
static_assert(WS_OFF_RAW % 16 == 0 && RAW_BYTES % 16 == 0 && WS_OFF_OFFS % 16 == 0, "raw buffers take bulk copies");
static_assert((NRAW & (NRAW - 1)) == 0, "raw buffers are indexed by j & (NRAW - 1)");
static_assert(WS_SH % QS == 0 && US == 2 * WS_SH, "a staging half holds whole quads");
static_assert(WS_E1 == 0 && WS_E2 == WS_E1 + 4, "epilogue-1 warps are 0..3 (TMEM lane quarter = warp)");
// named barriers (id, threads) of the groups
constexpr int NB_DEC = 1, NB_E1 = 2, NB_E2 = 3, NB_WO = 4;

CS_DEV bool grp_vote(int id, int n, bool ok)
{
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "bar.red.and.pred q, %2, %3, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(r)
        : "r"(ok ? 1u : 0u), "r"(id), "r"(n)
        : "memory");
    return r != 0;
}

template <bool PHASE, bool SCALE>
__global__ void __launch_bounds__(WS_THREADS, 1) k_fx_fstage_tc32ws(const __grid_constant__ Tc32Args args)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char* sm = smem_raw + ((1024u - (tc::smem_u32(smem_raw) & 1023u)) & 1023u);
    const uint32_t sbase = tc::smem_u32(sm);
    const CsFStageArgs& a = args.f;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tid = threadIdx.x;
    const uint32_t bar0 = sbase + WS_OFF_BAR;
    auto bar = [&](int i) { return bar0 + 8u * (uint32_t)i; };
    uint32_t* slot = reinterpret_cast<uint32_t*>(sm + WS_OFF_SLOT);
    int* offs = reinterpret_cast<int*>(sm + WS_OFF_OFFS);
    __half2* lut2 = reinterpret_cast<__half2*>(sm + WS_OFF_LUT);
    uint32_t* stg = reinterpret_cast<uint32_t*>(sm + WS_OFF_STG);

    for (int i = tid; i < CONST_BYTES / 16; i += WS_THREADS)
        reinterpret_cast<uint4*>(sm)[i] = __ldg(args.consts + i);
    for (int i = tid; i < 2 * A2P_REGION / 16; i += WS_THREADS)
        reinterpret_cast<uint4*>(sm + WS_OFF_A2P)[i] = make_uint4(0, 0, 0, 0);
    if (tid < 16) {
        const float l0 = a.lut[0], l1 = a.lut[1], l2 = a.lut[2], l3 = a.lut[3];
        auto lv = [&](int c) { return c == 0 ? l0 : c == 1 ? l1 : c == 2 ? l2 : l3; };
        lut2[tid] = __floats2half2_rn(lv(tid & 3), lv(tid >> 2));
    }
    if (tid == 0) {
        tc::mbar_init(bar(WB_B1FULL), 4);
        for (int b = 0; b < 2; b++) {
            tc::mbar_init(bar(WB_D1FULL + b), 1);
            tc::mbar_init(bar(WB_E1DONE + b), 4);
            tc::mbar_init(bar(WB_D2FULL + b), 1);
            tc::mbar_init(bar(WB_E2DONE + b), 4);
            tc::mbar_init(bar(WB_D2PFULL + b), 1);
        }
        tc::mbar_init(bar(WB_E2PDONE), 1);
        for (int t = 0; t < 2; t++) {
            tc::mbar_init(bar(WB_STGFULL + t), 4);
            tc::mbar_init(bar(WB_STGFREE + t), 4);
        }
        tc::mbar_init(bar(WB_DRAIN), 1);
        for (int r = 0; r < NRAW; r++) {
            tc::mbar_init(bar(WB_RAWFULL + r), 1);
            tc::mbar_init(bar(WB_RAWFREE + r), 4);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == WS_MMA) tc::tmem_alloc(tc::smem_u32(slot), TMEM_COLS);
    tc::fence_proxy_async();
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = *slot;

    const int64_t units = args.units;
    const int nunits = (blockIdx.x < units) ? (int)((units - 1 - blockIdx.x) / gridDim.x + 1) : 0;
    const int nquads = nunits * QUADS;
    const int K = a.K;
    auto unit_of = [&](int u, int& s, int& kb) {
        const uint32_t uu = blockIdx.x + (uint32_t)u * gridDim.x;
        const uint32_t si = uu / (uint32_t)args.units_k;
        s = (int)si;
        kb = (int)(uu - si * (uint32_t)args.units_k);
    };
    // a group leader's bounded wait (the group then votes on the outcome)
    auto lwait = [&](int i, uint32_t parity) {
        return tc::mbar_wait(bar(i), parity, &g_fst32_error, E_WORKER_WAIT, WAIT_CYCLES);
    };
    // channel-grouped k-blocked spectra: the 128-byte run of (channel c,
    // input s, 32-segment block kb), in runs of 64 halves
    __half* out = reinterpret_cast<__half*>(a.out);
    auto grun = [&](int c, int s, int kb) -> int64_t {
        return (((int64_t)(c >> 4) * args.s_rows + s) * args.nkb + kb) * 16 + (c & 15);
    };

    // epilogue-2 helpers: the delay phasor of input s_, segment k_ from channel
    // cstart in steps of cstep, and its product (and the channel scale) on X
#define TC32_PHASOR(s_, k_, cstart, cstep)                                              \
        float2 B = make_float2(1.f, 0.f), D = B;                                        \
        if (PHASE) {                                                                    \
            const int64_t sk = (int64_t)(s_) * K + (k_);                                \
            const float ph0 = __ldg(a.phase0 + sk), dph = __ldg(a.dphase + sk);         \
            float sn, cs;                                                               \
            sincosf(ph0 + (cstart) * dph, &sn, &cs);                                    \
            B = make_float2(cs, sn);                                                    \
            sincosf((cstep) * dph, &sn, &cs);                                           \
            D = make_float2(cs, sn);                                                    \
        }
#define TC32_APPLY(c_, X)                                                               \
        if (PHASE) {                                                                    \
            X = cmul(X, B);                                                             \
            B = cmul(B, D);                                                             \
        }                                                                               \
        if (SCALE) X = cscale(X, __ldg(scl + (c_)));
    if (warp == WS_MMA) {
        // ------------------------------ MMA issuer ------------------------------
        if (lane == 0) {
            const uint32_t id1 = tc::idesc_f16(128, 128, false, false, true);
            const uint32_t id2 = tc::idesc_f16(128, 64, false, false, false);
            auto w = [&](int i, uint32_t ph) {
                return tc::mbar_wait(bar(i), ph, &g_fst32_error, E_MMA_WAIT, WAIT_CYCLES);
            };
            // pass 1 of quad j: B1 -> D1[j & 1].  D1[j & 1] was last read by
            // epilogue 1 for quad j - 2, whose completion pass 2 of quad j - 2
            // waited for before this is issued.
            auto pass1 = [&](int j) -> bool {
                const int b = j & 1;
                if (!w(WB_B1FULL, (uint32_t)j & 1)) return false;
                tc::fence_after();
#pragma unroll
                for (int kk = 0; kk < 4; kk++) {
                    const uint64_t da = tc::smem_desc(sbase + OFF_A1 + 32u * kk, 16, 1024, tc::SW128);
                    const uint64_t db =
                        tc::smem_desc(sbase + WS_OFF_B1 + 2048u * kk, 8192, 1024, tc::SW128);
                    tc::mma_f16(tmem + COL_D1 + 128u * b, da, db, id1, kk ? 1u : 0u);
                }
                tc::commit(bar(WB_D1FULL + b));
                return true;
            };
            bool ok = nquads == 0 || pass1(0);
            for (int j = 0; ok && j < nquads; j++) {
                const int b = j & 1, u = j / QUADS;
                if (j + 1 < nquads && !pass1(j + 1)) break;
                if (j >= 2 && !w(WB_E2DONE + b, (uint32_t)((j - 2) >> 1) & 1)) break;   // D2[b] read
                if (!w(WB_E1DONE + b, (uint32_t)(j >> 1) & 1)) break;                  // A2[b] written, D1[b] read
                tc::fence_after();
#pragma unroll
                for (int kk = 0; kk < 4; kk++) {
                    const uint64_t da =
                        tc::smem_desc(sbase + WS_OFF_A2 + (uint32_t)b * A2_BYTES + 32u * kk, 16, 1024, tc::SW128);
                    const uint64_t db = tc::smem_desc(sbase + OFF_B2 + 32u * kk, 16, 1024, tc::SW128);
                    tc::mma_f16(tmem + COL_D2 + 64u * b, da, db, id2, kk ? 1u : 0u);
                }
                tc::commit(bar(WB_D2FULL + b));
                if (j % QUADS == QUADS - 1) {
                    if (u >= 1 && !w(WB_E2PDONE, (uint32_t)(u - 1) & 1)) break;       // D2' read
                    tc::fence_after();
#pragma unroll
                    for (int kk = 0; kk < 4; kk++) {
                        const uint64_t da = tc::smem_desc(
                            sbase + WS_OFF_A2P + (uint32_t)(u & 1) * A2P_REGION + 32u * kk, 16, 1024, tc::SW128);
                        const uint64_t db = tc::smem_desc(sbase + OFF_B2 + 32u * kk, 16, 1024, tc::SW128);
                        tc::mma_f16(tmem + COL_D2P, da, db, id2, kk ? 1u : 0u);
                    }
                    tc::commit(bar(WB_D2PFULL + (u & 1)));
                }
            }
            tc::commit(bar(WB_DRAIN));
            tc::mbar_wait(bar(WB_DRAIN), 0, &g_fst32_error, E_MMA_WAIT, WAIT_CYCLES);
        }
        __syncwarp();
    } else if (warp < WS_E2) {
        // ------------------------------ epilogue 1 ------------------------------
        const int q = warp, gt = tid;                       // group thread 0..127
        const bool leader = gt == 0;
        const int k1 = 8 * q + (lane >> 2);
        float2 tw[4][2];
#pragma unroll
        for (int m = 0; m < 4; m++)
#pragma unroll
            for (int e = 0; e < 2; e++) {
                const int n2 = 8 * m + 2 * (lane & 3) + e;
                float sn, cs;
                sincospif(-(float)((n2 * k1) & 2047) / 1024.0f, &sn, &cs);
                tw[m][e] = make_float2(cs, sn);
            }
        const uint32_t e1base = sw128(k1, 2 * (lane & 3));   // row 32 h + k1: + 4096 h
        const int m32 = (lane >> 2) & 3, e32 = lane >> 4;
        const int n2_32 = 8 * m32 + 2 * (lane & 3) + e32;
        float2 tw32;
        {
            float sn, cs;
            sincospif(-(float)n2_32 / 32.0f, &sn, &cs);
            tw32 = make_float2(cs, sn);
        }
        for (int j = 0; j < nquads; j++) {
            const int b = j & 1, qd = j % QUADS, u = j / QUADS;
            bool ok = true;
            if (leader) {
                // A2' region u & 1 read by pass 2' of unit u - 2; A2[b] read by
                // pass 2 of quad j - 2; D1[b] of quad j written
                if (qd == 0 && u >= 2) ok = lwait(WB_D2PFULL + (u & 1), (uint32_t)((u - 2) >> 1) & 1);
                if (ok && j >= 2) ok = lwait(WB_D2FULL + b, (uint32_t)((j - 2) >> 1) & 1);
                if (ok) ok = lwait(WB_D1FULL + b, (uint32_t)(j >> 1) & 1);
            }
            if (!grp_vote(NB_E1, 128, ok)) break;
            tc::fence_after();
            unsigned char* a2 = sm + WS_OFF_A2 + b * A2_BYTES;
            unsigned char* a2p = sm + WS_OFF_A2P + (u & 1) * A2P_REGION;
            auto e1seg = [&](int h, const uint32_t (&r)[16]) {
                unsigned char* a2h = a2 + 4096 * h;
#pragma unroll
                for (int m = 0; m < 4; m++) {
                    const float2 y0 = make_float2(__uint_as_float(r[4 * m]), __uint_as_float(r[4 * m + 2]));
                    const float2 y1 = make_float2(__uint_as_float(r[4 * m + 1]), __uint_as_float(r[4 * m + 3]));
                    const float2 z0 = cmul(y0, tw[m][0]), z1 = cmul(y1, tw[m][1]);
                    *reinterpret_cast<uint32_t*>(a2h + (e1base ^ (m << 4))) = h2u(__floats2half2_rn(z0.x, z1.x));
                    *reinterpret_cast<uint32_t*>(a2h + (e1base ^ (m << 4) ^ 64u)) = h2u(__floats2half2_rn(z0.y, z1.y));
                }
            };
            // the real k1 = 32 row (TMEM lanes 16..23 of this warp's quarter) of segment h
            // -> row 4 qd + h of the unit's A2' region
            auto e1row32 = [&](int h, const uint32_t (&r32)[16]) {
                const bool mb1 = m32 & 1, mb2 = m32 & 2;
                const uint32_t ya = mb2 ? (mb1 ? r32[12] : r32[8]) : (mb1 ? r32[4] : r32[0]);
                const uint32_t yb = mb2 ? (mb1 ? r32[13] : r32[9]) : (mb1 ? r32[5] : r32[1]);
                const float y = __uint_as_float(e32 ? yb : ya);
                const uint32_t prow = QS * qd + h;
                *reinterpret_cast<__half*>(a2p + sw128(prow, n2_32)) = __float2half_rn(y * tw32.x);
                *reinterpret_cast<__half*>(a2p + sw128(prow, 32 + n2_32)) = __float2half_rn(y * tw32.y);
            };
            // two segments per TMEM wait
#pragma unroll 1
            for (int h = 0; h < QS; h += 2) {
                const uint32_t d1 = tmem + COL_D1 + 128u * b + 32u * h;
                uint32_t r0[16], r1[16];
                tc::tmem_ld_16x256b_x4(d1 + ((uint32_t)(32 * q) << 16), r0);
                tc::tmem_ld_16x256b_x4(d1 + 32u + ((uint32_t)(32 * q) << 16), r1);
                if ((q & ~1) == h) {
                    // this warp's share of the k1 = 32 row: segment q, from the
                    // copy of the row in its own lane quarter (rows 32 q + 16..23)
                    uint32_t s0[16];
                    tc::tmem_ld_16x256b_x4(d1 + 32u * (q & 1) + ((uint32_t)(32 * q + 16) << 16), s0);
                    tc::tmem_ld_wait();
                    pin16(r0);
                    pin16(r1);
                    pin16(s0);
                    e1row32(q, s0);
                } else {
                    tc::tmem_ld_wait();
                    pin16(r0);
                    pin16(r1);
                }
                e1seg(h, r0);
                e1seg(h + 1, r1);
            }
            tc::fence_before();
            tc::fence_proxy_async();
            warp_arrive(bar(WB_E1DONE + b));
        }
    } else if (warp < WS_DEC) {
        // ------------------------------ epilogue 2 ------------------------------
        const int q = warp & 3, gt = tid - 32 * WS_E2;
        const bool leader = gt == 0;
        const int kk1 = lane;
        for (int j = 0; j < nquads; j++) {
            const int b = j & 1, qd = j % QUADS, u = j / QUADS, t = j / (WS_SH / QS), sh = t & 1;
            int s, kb;
            unit_of(u, s, kb);
            const float* scl = SCALE ? a.scale + (int64_t)s * FC : nullptr;
            bool ok = true;
            if (leader) {
                // staging half sh drained (for the unit before); D2[b] of quad j written
                if (j % (WS_SH / QS) == 0 && t >= 2) ok = lwait(WB_STGFREE + sh, (uint32_t)((t >> 1) - 1) & 1);
                if (ok) ok = lwait(WB_D2FULL + b, (uint32_t)(j >> 1) & 1);
            }
            if (!grp_vote(NB_E2, 128, ok)) break;
            tc::fence_after();
            const int seg = QS * qd + q, k = kb * US + seg;
            uint32_t* srow = stg + seg * WS_STG_PITCH;
            const uint32_t d2 = tmem + COL_D2 + 64u * b + ((uint32_t)(32 * q) << 16);
            // k2 blocks h = 0..3 in two pairs, one TMEM wait per pair
            auto e2blk = [&](int h, const uint32_t (&re)[8], const uint32_t (&im)[8]) {
                if (h < 2) {
                    const int c0 = kk1 + 512 * h;
                    TC32_PHASOR(s, k, (float)c0, 64.f)
#pragma unroll
                    for (int i = 0; i < 8; i++) {
                        float2 X = make_float2(__uint_as_float(re[i]), __uint_as_float(im[i]));
                        TC32_APPLY(c0 + 64 * i, X)
                        srow[c0 + 64 * i] = h2u(__floats2half2_rn(X.x, X.y));
                    }
                } else if (kk1 > 0) {
                    const int c0 = FC - kk1 - 512 * (h - 2);
                    TC32_PHASOR(s, k, (float)c0, -64.f)
#pragma unroll
                    for (int i = 0; i < 8; i++) {
                        float2 X = make_float2(__uint_as_float(re[i]), -__uint_as_float(im[i]));
                        TC32_APPLY(c0 - 64 * i, X)
                        srow[c0 - 64 * i] = h2u(__floats2half2_rn(X.x, X.y));
                    }
                }
            };
#pragma unroll 1
            for (int h = 0; h < 4; h += 2) {
                uint32_t re0[8], im0[8], re1[8], im1[8];
                tc::tmem_ld_32x32b_x8(d2 + 8u * h, re0);
                tc::tmem_ld_32x32b_x8(d2 + 32u + 8u * h, im0);
                tc::tmem_ld_32x32b_x8(d2 + 8u * (h + 1), re1);
                tc::tmem_ld_32x32b_x8(d2 + 32u + 8u * (h + 1), im1);
                tc::tmem_ld_wait();
#pragma unroll
                for (int i = 0; i < 8; i++) asm volatile("" : "+r"(re0[i]), "+r"(im0[i]), "+r"(re1[i]), "+r"(im1[i]));
                e2blk(h, re0, im0);
                e2blk(h + 1, re1, im1);
            }
            tc::fence_before();
            warp_arrive(bar(WB_E2DONE + b));
            if (j % (WS_SH / QS) == WS_SH / QS - 1) warp_arrive(bar(WB_STGFULL + sh));
        }
    } else if (warp < WS_WO) {
        // ------------------------------ decode ------------------------------
        const int gt = tid - 32 * WS_DEC;                   // 0..127
        const bool leader = gt == 0;
        // Thread gt decodes raw word wd (16 samples: n1 = wd / 2, n2 = 16 (wd & 1)
        // + 0..15).  The order puts eight consecutive lanes on eight rows n1 of
        // one n2 half, so each quarter-warp's 16-byte B1 stores hit eight
        // different swizzled chunks (no bank conflict).
        const int wd = ((gt & 7) << 1) | ((gt >> 3) & 1) | (gt & ~15);
        // the four levels as FP16 bytes 0-7 of {t1:t0}; code c is bytes 2c, 2c + 1
        const uint32_t t0 = h2u(lut2[4]), t1 = h2u(lut2[14]);
        for (int j = 0; j < nquads; j++) {
            const int buf = j & (NRAW - 1);
            // raw words of quad j landed, and B1 free (pass 1 of quad j - 1 done)
            bool ok = true;
            if (leader) {
                ok = lwait(WB_RAWFULL + buf, (uint32_t)(j / NRAW) & 1);
                if (ok && j > 0) ok = lwait(WB_D1FULL + ((j - 1) & 1), (uint32_t)((j - 1) >> 1) & 1);
            }
            if (!grp_vote(NB_DEC, 128, ok)) break;
            const uint32_t* rw0 = reinterpret_cast<const uint32_t*>(sm + WS_OFF_RAW + buf * RAW_BYTES);
            const int4 o4 = *reinterpret_cast<const int4*>(offs + buf * QS);
            const int ov[QS] = {o4.x, o4.y, o4.z, o4.w};
            // every load of the quad before any store (the B1 stores could
            // otherwise alias them and serialise the segments)
            uint32_t bits[QS];
#pragma unroll
            for (int g = 0; g < QS; g++) {                  // segment g of the quad, word wd
                const uint32_t* rw = rw0 + g * RAWC * 4 + (ov[g] >> 4) + wd;
                bits[g] = __funnelshift_r(rw[0], rw[1], 2 * (ov[g] & 15));
            }
            // word w of the 8 output words holds samples 2w, 2w + 1 (codes a, b):
            // a byte_perm of {t1:t0} with selector nibbles 2a, 2a + 1, 2b, 2b + 1
            // = 0x1010 + 34 a + 8704 b.  Words w and w + 4 share one selector
            // computation, one per 16-bit half (no carry: the sum stays below 2^15).
            uint32_t hv[QS][8];
#pragma unroll
            for (int g = 0; g < QS; g++)
#pragma unroll
                for (int w = 0; w < 4; w++) {
                    const uint32_t pa = (bits[g] >> (4 * w)) & 0x00030003u;
                    const uint32_t pb = (bits[g] >> (4 * w + 2)) & 0x00030003u;
                    const uint32_t sel = pa * 34u + pb * 8704u + 0x10101010u;
                    hv[g][w] = __byte_perm(t0, t1, sel);
                    hv[g][w + 4] = __byte_perm(t0, t1, sel >> 16);
                }
            warp_arrive(bar(WB_RAWFREE + buf));            // this warp's reads of the buffer are done
            unsigned char* b1 = sm + WS_OFF_B1;
            const int n1 = wd >> 1;
#pragma unroll
            for (int g = 0; g < QS; g++) {
                const int chunk = 4 * (g & 1) + 2 * (wd & 1);
                unsigned char* rowp = b1 + (g >> 1) * 8192 + n1 * 128;
                *reinterpret_cast<uint4*>(rowp + (((chunk ^ n1) & 7) << 4)) =
                    make_uint4(hv[g][0], hv[g][1], hv[g][2], hv[g][3]);
                *reinterpret_cast<uint4*>(rowp + ((((chunk + 1) ^ n1) & 7) << 4)) =
                    make_uint4(hv[g][4], hv[g][5], hv[g][6], hv[g][7]);
            }
            tc::fence_proxy_async();
            warp_arrive(bar(WB_B1FULL));
        }
    } else if (warp < WS_MMA) {
        // ------------------------------ write-out ------------------------------
        // staging half t & 1 of unit t / 2: per channel the 16 segments' Re
        // and Im halves; lanes 2i, 2i + 1 take segments 0-7 and 8-15 of one
        // channel, so each plane's 32 bytes leave as one whole sector
        const int gt = tid - 32 * WS_WO;                    // 0..127
        const bool leader = gt == 0;
        const int nhalves = 2 * nunits;
        bool kfail = false;                                 // warp WS_WO: a pass-2' wait failed
        for (int t = 0; t < nhalves; t++) {
            const int sh = t & 1, u = t >> 1;
            int s, kb;
            unit_of(u, s, kb);
            bool ok = !kfail;
            if (leader && ok) ok = lwait(WB_STGFULL + sh, (uint32_t)(t >> 1) & 1);
            if (!grp_vote(NB_WO, 128, ok)) break;
            __half* o = out + WS_SH * sh;
#pragma unroll 2
            for (int r = 0; r < 2 * FC / 128; r++) {
                const int task = r * 128 + gt;
                const int c = task >> 1, g8 = task & 1;
                if ((c & 63) == 32) continue;               // the k1 = 32 channels: below
                const uint32_t* col = stg + (WS_SH * sh + 8 * g8) * WS_STG_PITCH + c;
                uint32_t w[8];
#pragma unroll
                for (int i = 0; i < 8; i++) w[i] = col[i * WS_STG_PITCH];
                __half* run = o + grun(c, s, kb) * 64 + 8 * g8;
                *reinterpret_cast<uint4*>(run) =
                    make_uint4(__byte_perm(w[0], w[1], 0x5410), __byte_perm(w[2], w[3], 0x5410),
                               __byte_perm(w[4], w[5], 0x5410), __byte_perm(w[6], w[7], 0x5410));
                *reinterpret_cast<uint4*>(run + 32) =
                    make_uint4(__byte_perm(w[0], w[1], 0x7632), __byte_perm(w[2], w[3], 0x7632),
                               __byte_perm(w[4], w[5], 0x7632), __byte_perm(w[6], w[7], 0x7632));
            }
            warp_arrive(bar(WB_STGFREE + sh));
            if (sh == 1 && warp == WS_WO) {
                // the unit's k1 = 32 channels c = 32 + 64 k2 from pass 2': this
                // warp (lane quarter 0, lane = segment) writes them to the spectra
                // directly, each store a channel's 32 segments of one plane (64 B)
                bool okp = true;
                if (lane == 0) okp = lwait(WB_D2PFULL + (u & 1), (uint32_t)(u >> 1) & 1);
                if (!__shfl_sync(0xffffffffu, okp, 0)) {
                    kfail = true;
                } else {
                    tc::fence_after();
                    const float* scl = SCALE ? a.scale + (int64_t)s * FC : nullptr;
                    __half* o = out + lane;
                    const int kq = kb * US + lane;
#pragma unroll 1
                    for (int h = 0; h < 2; h++) {
                        uint32_t re[8], im[8];
                        tc::tmem_ld_32x32b_x8(tmem + COL_D2P + 8u * h, re);
                        tc::tmem_ld_32x32b_x8(tmem + COL_D2P + 32u + 8u * h, im);
                        tc::tmem_ld_wait();
#pragma unroll
                        for (int i = 0; i < 8; i++) asm volatile("" : "+r"(re[i]), "+r"(im[i]));
                        const int c0 = 32 + 512 * h;
                        TC32_PHASOR(s, kq, (float)c0, 64.f)
#pragma unroll
                        for (int i = 0; i < 8; i++) {
                            const int c = c0 + 64 * i;
                            float2 X = make_float2(__uint_as_float(re[i]), __uint_as_float(im[i]));
                            TC32_APPLY(c, X)
                            __half* oc = o + grun(c, s, kb) * 64;
                            oc[0] = __float2half_rn(X.x);
                            oc[32] = __float2half_rn(X.y);
                        }
                    }
                    tc::fence_before();
                    warp_arrive(bar(WB_E2PDONE));
                }
            }
        }
    } else if (warp == WS_FETCH) {
        // ------------------------------ raw fetch ------------------------------
        // Raw words of quad j into buffer j & (NRAW - 1): lane g < QS copies
        // segment g's RAWC chunks with one bulk copy (the part inside the
        // input; chunks outside it are zeroed, as the lockstep form's
        // zero-filled cp.async leaves them) and the buffer's barrier completes
        // when all bytes have landed.
        const int64_t chunks = a.bytes_per_input >> 4;
        int issued = 0;
        for (int j = 0; j < nquads; j++) {
            const int buf = j & (NRAW - 1);
            bool ok = true;
            if (lane == 0 && j >= NRAW) ok = lwait(WB_RAWFREE + buf, (uint32_t)(j / NRAW - 1) & 1);
            if (!__shfl_sync(0xffffffffu, ok, 0)) break;
            int s, kb;
            unit_of(j / QUADS, s, kb);
            const uint32_t rb = bar(WB_RAWFULL + buf);
            int64_t ci0 = 0;
            int lo = 0, hi = 0;
            if (lane < QS) {
                const int k = kb * US + (j % QUADS) * QS + lane;
                const int64_t start = a.start_sample + (int64_t)k * FN + (a.shift ? __ldg(a.shift + (int64_t)s * K + k) : 0);
                ci0 = start >> 6;
                const int64_t l = -ci0 < 0 ? 0 : -ci0, h = chunks - ci0;
                lo = (int)(l < RAWC ? l : RAWC);
                hi = (int)(h < lo ? lo : h < RAWC ? h : RAWC);
                offs[buf * QS + lane] = (int)(start & 63);
                unsigned char* seg = sm + WS_OFF_RAW + buf * RAW_BYTES + lane * RAWC * 16;
                for (int c = 0; c < lo; c++) *reinterpret_cast<uint4*>(seg + 16 * c) = make_uint4(0, 0, 0, 0);
                for (int c = hi; c < RAWC; c++) *reinterpret_cast<uint4*>(seg + 16 * c) = make_uint4(0, 0, 0, 0);
            }
            uint32_t total = 16u * (uint32_t)(hi - lo);
            total += __shfl_xor_sync(0xffffffffu, total, 1);
            total += __shfl_xor_sync(0xffffffffu, total, 2);
            __syncwarp();
            if (lane == 0) tc::mbar_expect_tx(rb, total);   // the phase's one arrival
            __syncwarp();
            if (lane < QS && hi > lo)
                tc::bulk_load(sbase + WS_OFF_RAW + buf * RAW_BYTES + (lane * RAWC + lo) * 16,
                              a.raw + (int64_t)s * a.bytes_per_input + 16 * (ci0 + lo), 16u * (uint32_t)(hi - lo), rb);
            issued = j + 1;
        }
        // copies still in flight (the latest phase of each buffer) land before the CTA ends
        if (lane == 0)
            for (int q = issued > NRAW ? issued - NRAW : 0; q < issued; q++)
                lwait(WB_RAWFULL + (q & (NRAW - 1)), (uint32_t)(q / NRAW) & 1);
        __syncwarp();
    }
#undef TC32_PHASOR
#undef TC32_APPLY
    tc::fence_before();
    __syncthreads();
    if (warp == WS_MMA) {
        tc::fence_after();
        tc::tmem_dealloc(tmem, TMEM_COLS);
    }
}

// A1 (DFT-64: per TMEM lane quarter q the Re rows 32q..32q+7 and Im rows
// 32q+8..32q+15 of k1 = 8q..8q+7; rows 16..23 the real k1 = 32 row) and B2
// (DFT-32 as a real 64 x 64 operand: rows k2 give Re X, rows 32 + k2 Im X) in
// FP16, 128-byte-swizzled K-major, one copy per device.
std::mutex g_const_mu;
std::map<int, uint4*> g_consts;

const uint4* tc32_constants()
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    std::lock_guard<std::mutex> lk(g_const_mu);
    auto it = g_consts.find(dev);
    if (it != g_consts.end()) return it->second;
    std::vector<__half> h(CONST_BYTES / 2, __float2half(0.f));
    auto put = [&](int base, int row, int k, double v) {
        const uint32_t off = (uint32_t)row * 128 + ((((k >> 3) ^ row) & 7) << 4) + (k & 7) * 2;
        h[(base + off) / 2] = __double2half(v);
    };
    for (int r = 0; r < 128; r++) {
        const int q = r / 32, rr = r % 32;
        for (int n1 = 0; n1 < 64; n1++) {
            double v = 0.0;
            if (rr < 16) {
                const int k1 = 8 * q + rr % 8;
                const double th = 2.0 * M_PI * (double)((n1 * k1) % 64) / 64.0;
                v = rr < 8 ? std::cos(th) : -std::sin(th);
            } else if (rr < 24) {
                // W_64^(32 n1): the real k1 = 32 row, in every lane quarter (the
                // lockstep form reads quarter 0's; the warp-specialised form's
                // epilogue-1 warp q reads quarter q's for segment q of a quad)
                v = (n1 & 1) ? -1.0 : 1.0;
            }
            put(OFF_A1, r, n1, v);
        }
    }
    for (int r = 0; r < 64; r++) {
        const int k2 = r % 32, part = r / 32;
        for (int kk = 0; kk < 64; kk++) {
            const int plane = kk / 32, n2 = kk % 32;
            const double th = 2.0 * M_PI * (double)((n2 * k2) % 32) / 32.0;
            const double c = std::cos(th), sn = std::sin(th);
            // Re X = sum Zr cos + Zi sin;  Im X = sum -Zr sin + Zi cos
            const double v = part == 0 ? (plane == 0 ? c : sn) : (plane == 0 ? -sn : c);
            put(OFF_B2, r, kk, v);
        }
    }
    uint4* d = nullptr;
    if (cudaMalloc(&d, CONST_BYTES) != cudaSuccess) return nullptr;
    if (cudaMemcpy(d, h.data(), CONST_BYTES, cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(d);
        return nullptr;
    }
    g_consts[dev] = d;
    return d;
}

int g_sms32 = 0;

}  // namespace

bool cs_fstage_tc32_supported(const CsFStageArgs& a)
{
    const int kp = a.kp ? a.kp : a.K;
    return a.N == FN && a.format == CS_SPECTRA_F16 && !a.msb_first && !a.seg_major && a.kblock && a.K % US == 0 &&
           kp % US == 0;
}

int cs_fx_fstage_tc32(const CsFStageArgs& a, cudaStream_t st, bool specialised)
{
    if (!cs_fstage_tc32_supported(a)) return CS_ERR_UNSUPPORTED;
    // the warp-specialised form writes the channel-grouped layout, the lockstep form layout 1
    if (a.kblock != (specialised ? 2 : 1)) return CS_ERR_ARG;
    if ((int64_t)a.S * (a.K / US) >= (int64_t)1 << 31) return CS_ERR_UNSUPPORTED;   // unit indices are 32-bit
    if (!a.raw || !a.out || a.S <= 0 || a.K <= 0) return CS_ERR_ARG;
    if ((uintptr_t)a.raw % 16 || a.bytes_per_input % 16 || (uintptr_t)a.out % 16) return CS_ERR_ARG;
    const uint4* consts = tc32_constants();
    if (!consts) return (int)cudaErrorMemoryAllocation;
    if (!g_sms32) {
        int dev = 0, n = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        g_sms32 = n > 0 ? n : 148;
    }
    void* errp = nullptr;
    CS_CUDA_TRY(cudaGetSymbolAddress(&errp, g_fst32_error));
    CS_CUDA_TRY(cudaMemsetAsync(errp, 0, sizeof(unsigned), st));
    Tc32Args t{};
    t.f = a;
    t.consts = consts;
    t.units_k = a.K / US;
    t.units = (int64_t)a.S * t.units_k;
    t.nkb = (a.kp ? a.kp : a.K) / US;
    t.s_rows = a.S_out ? a.S_out : a.S;
    const int grid = (int)std::min<int64_t>(t.units, g_sms32);
    // the delay phasor and the channel scale are compiled in only where used;
    // specialised: the warp-specialised form
    if (specialised) {
        auto kern = a.phase0 ? (a.scale ? k_fx_fstage_tc32ws<true, true> : k_fx_fstage_tc32ws<true, false>)
                             : (a.scale ? k_fx_fstage_tc32ws<false, true> : k_fx_fstage_tc32ws<false, false>);
        CS_CUDA_TRY(cs_smem_at_least(reinterpret_cast<const void*>(kern), (int)(WS_SMEM_BYTES)));
        kern<<<grid, WS_THREADS, WS_SMEM_BYTES, st>>>(t), cs_count_launches(1);
    } else {
        auto kern = a.phase0 ? (a.scale ? k_fx_fstage_tc32<true, true> : k_fx_fstage_tc32<true, false>)
                             : (a.scale ? k_fx_fstage_tc32<false, true> : k_fx_fstage_tc32<false, false>);
        CS_CUDA_TRY(cs_smem_at_least(reinterpret_cast<const void*>(kern), (int)(SMEM_BYTES)));
        kern<<<grid, THREADS, SMEM_BYTES, st>>>(t), cs_count_launches(1);
    }
    return (int)cudaGetLastError();
}

int cs_fstage_tc32_status(unsigned* code)
{
    return (int)cudaMemcpyFromSymbol(code, g_fst32_error, sizeof(unsigned));
}
