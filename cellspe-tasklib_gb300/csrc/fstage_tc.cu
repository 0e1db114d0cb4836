// K-b/K-c on the tensor cores: the FX F stage for N = 2048 with FP16 spectra
// out (the input of the tcgen05 X stage).
//
// The real 2048-point DFT X[c] = sum_n x[n] W_2048^(n c), c < 1024, runs as a
// four-step transform with both passes on the tensor cores (FP16 operands,
// FP32 accumulators in TMEM).  With n = n2 + 32 n1 and c = k1 + 64 k2:
//     Y[k1][n2] = sum_n1 x[n2 + 32 n1] W_64^(n1 k1)          (pass 1, real in)
//     Z[k1][n2] = Y[k1][n2] W_2048^(n2 k1)                   (CUDA cores)
//     X[k1 + 64 k2] = sum_n2 Z[k1][n2] W_32^(n2 k2)          (pass 2, k2 < 16)
// Pass 1 is D1 = A1 . B1 with A1 the constant DFT-64 matrix (128 rows: Re and
// Im of Y[k1], k1 < 64, ordered so that rows 16g..16g+7 hold Re and rows
// 16g+8..16g+15 hold Im of k1 = 8g..8g+7) and B1 the unpacked samples of 8
// segments in their natural order, which is the MN-major layout of a
// K = n1 (64) x N = (segment, n2) (256) operand.  A 16x256b TMEM load then
// gives each thread Re and Im of the same Y values, so the twiddle needs no
// data exchange.  Pass 2 is D2 = A2 . B2 per pair of segments: A2 rows are
// (segment, k1), K = (Re Z[n2], Im Z[n2]); B2 is the constant DFT-32 matrix
// as a real 32 x 64 operand (rows 0..15 give Re X[k2], 16..31 Im X[k2]).
// The epilogue applies the fringe / fractional-delay phasor and the optional
// channel scale, casts to FP16 and writes the spectra corner-turned
// (__half [C][2][S][K]) as the CUDA-core F stage does.
//
// Warp roles: warps 0..7 (workers) fetch raw words (cp.async), unpack,
// run both epilogues and repack the unit's spectra for the write-out; warp 8
// owns TMEM and one thread issues the MMAs; one thread of warp 9 writes the
// repacked spectra with TMA stores (3D boxes of 256 output rows x 8
// segments) and releases the buffer once it has been read.  Work unit = 8 consecutive segments of one input; CTAs are
// persistent and walk units blockIdx.x, +gridDim.x, ...  Unpacking unit j+1
// overlaps pass 2 of unit j; pass 1 of unit j+1 overlaps the second
// epilogue and the write-out of unit j.  Every mbarrier wait is bounded (~2 s): on timeout the
// threads record an error code, leave their loops together (worker votes),
// drain the tensor pipe and free TMEM.
#include "common.cuh"
#include "kernels.h"
#include "tcgen05.cuh"
#include "tma.h"

#include <cuda_fp16.h>

#include <map>
#include <mutex>
#include <vector>

namespace {

constexpr int FN = 2048, FC = 1024, G = 8;            // segments per unit
constexpr int WORKERS = 256, THREADS = WORKERS + 64;    // + MMA warp (8) + store warp (9)
constexpr int RAWC = 34;                              // 16-byte raw chunks per segment (2048 samples + slack)
constexpr int OFF_A1 = 0;                             // DFT-64, 128 rows x 128 B, K-major, 128-byte swizzle
constexpr int OFF_B2 = 16384;                         // DFT-32, 32 rows x 128 B
constexpr int CONST_BYTES = 20480;
constexpr int OFF_B1 = 20480;                         // samples: 2 buffers x 4 atoms x (64 rows x 128 B)
constexpr int B1_BYTES = 32768;
constexpr int OFF_A2 = OFF_B1 + 2 * B1_BYTES;         // Z: 4 tiles x (128 rows x 128 B)
constexpr int A2_TILE = 16384;
constexpr int OFF_STG = OFF_A2 + 4 * A2_TILE;         // staging: [FC][G+1] half2
constexpr int STG_BYTES = FC * (G + 1) * 4;
constexpr int OFF_RAW = OFF_STG + STG_BYTES;          // 2 x G x RAWC x 16
constexpr int RAW_BYTES = G * RAWC * 16;
constexpr int OFF_OFFS = OFF_RAW + 2 * RAW_BYTES;     // sample offsets: 2 x G ints
constexpr int OFF_LUT = OFF_OFFS + 64;                // 16 half2 pair levels
constexpr int OFF_BAR = OFF_LUT + 64;                 // mbarriers
constexpr int NBAR = 10;
constexpr int OFF_SLOT = OFF_BAR + 8 * NBAR;
constexpr int SMEM_USED = OFF_SLOT + 16;
constexpr int SMEM_BYTES = SMEM_USED + 1024;          // + alignment of the base to 1024 B
constexpr uint32_t TMEM_COLS = 512;                   // D1: 0..255, D2 tiles: 256 + 32 t
constexpr long long WAIT_CYCLES = 4000000000LL;       // ~2 s

// barrier indices
constexpr int B_B1FULL0 = 0, B_B1FULL1 = 1, B_D1FULL = 2, B_EPI1 = 3, B_D2FULL = 4, B_EPI2 = 5, B_DRAIN = 6,
              B_REPACK = 7, B_STORED = 8;
// error codes
constexpr unsigned E_MMA_WAIT = 1, E_WORKER_WAIT = 2, E_STORE_WAIT = 3;

__device__ unsigned g_fstc_error;

static_assert(SMEM_BYTES <= 227 * 1024, "shared memory");

CS_DEV void cp_async16(uint32_t dst, const void* src, bool valid)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(valid ? 16 : 0)
                 : "memory");
}
CS_DEV void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
CS_DEV void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

CS_DEV void worker_bar() { asm volatile("bar.sync 1, 256;" ::: "memory"); }
// all 256 workers agree on `ok` (and synchronise)
CS_DEV bool worker_vote(bool ok)
{
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "bar.red.and.pred q, 1, 256, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(r)
        : "r"(ok ? 1u : 0u)
        : "memory");
    return r != 0;
}

// After tcgen05.wait::ld: ties the loaded registers to that point so that no
// use can be scheduled above the wait.
CS_DEV void pin16(uint32_t (&r)[16])
{
#pragma unroll
    for (int i = 0; i < 16; i++) asm volatile("" : "+r"(r[i]));
}

// TMA store of one box from shared memory (bulk-group completion)
CS_DEV void tma_store_3d(uint32_t src, const CUtensorMap* tm, int x, int y, int z)
{
    asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.bulk_group [%0, {%1, %2, %3}], [%4];"
                 ::"l"(reinterpret_cast<uint64_t>(tm)), "r"(x), "r"(y), "r"(z), "r"(src)
                 : "memory");
}
CS_DEV void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// the source shared memory of every committed bulk store has been read
CS_DEV void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
// every committed bulk store has completed
CS_DEV void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// byte offset of element (row, k) of a 128-byte-swizzled K-major operand
// (rows of 64 FP16, 8-row groups every 1024 B)
CS_DEV uint32_t sw128(uint32_t row, uint32_t k)
{
    return row * 128 + ((((k >> 3) ^ row) & 7) << 4) + (k & 7) * 2;
}

struct TcFArgs {
    CsFStageArgs f;
    const uint4* consts;      // A1 + B2, CONST_BYTES, already swizzled
    int units_k;              // units per input = ceil(K / 8)
    int64_t units;            // S * units_k
};

template <bool PHASE>
__global__ void __launch_bounds__(THREADS, 1) k_fx_fstage_tc(const __grid_constant__ TcFArgs args,
                                                                const __grid_constant__ CUtensorMap tmap_out)
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

    // constants into shared memory, barriers, TMEM
    for (int i = tid; i < CONST_BYTES / 16; i += THREADS)
        reinterpret_cast<uint4*>(sm)[i] = __ldg(args.consts + i);
    if (tid < 16) lut2[tid] = __floats2half2_rn(a.lut[tid & 3], a.lut[tid >> 2]);
    if (tid == 0) {
        tc::mbar_init(bar(B_B1FULL0), WORKERS);
        tc::mbar_init(bar(B_B1FULL1), WORKERS);
        tc::mbar_init(bar(B_D1FULL), 1);
        tc::mbar_init(bar(B_EPI1), WORKERS);
        tc::mbar_init(bar(B_D2FULL), 1);
        tc::mbar_init(bar(B_EPI2), WORKERS);
        tc::mbar_init(bar(B_DRAIN), 1);
        tc::mbar_init(bar(B_REPACK), WORKERS);
        tc::mbar_init(bar(B_STORED), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 8) tc::tmem_alloc(tc::smem_u32(slot), TMEM_COLS);
    tc::fence_proxy_async();                       // constant operands -> tensor core
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = *slot;

    const int64_t units = args.units;
    const int nunits = (blockIdx.x < units) ? (int)((units - 1 - blockIdx.x) / gridDim.x + 1) : 0;
    const int S = a.S, K = a.K;

    if (warp == 8) {
        // ------------------------------ MMA issuer ------------------------------
        if (lane == 0) {
            const uint32_t id1 = tc::idesc_f16(128, 256, false, false, true);    // B1 MN-major
            const uint32_t id2 = tc::idesc_f16(128, 32, false, false, false);
            bool ok = true;
            for (int j = 0; j < nunits && ok; j++) {
                ok = tc::mbar_wait(bar(j & 1), (uint32_t)(j >> 1) & 1, &g_fstc_error, E_MMA_WAIT, WAIT_CYCLES);
                if (ok && j > 0)
                    ok = tc::mbar_wait(bar(B_EPI1), (uint32_t)(j - 1) & 1, &g_fstc_error, E_MMA_WAIT, WAIT_CYCLES);
                if (!ok) break;
                tc::fence_after();
                const uint32_t b1 = sbase + OFF_B1 + (uint32_t)(j & 1) * B1_BYTES;
#pragma unroll
                for (int kk = 0; kk < 4; kk++) {
                    const uint64_t da = tc::smem_desc(sbase + OFF_A1 + 32u * kk, 16, 1024, tc::SW128);
                    // MN-major: 8-row K groups every 1024 B, 64-wide N atoms every 8192 B
                    const uint64_t db = tc::smem_desc(b1 + 2048u * kk, 8192, 1024, tc::SW128);
                    tc::mma_f16(tmem, da, db, id1, kk ? 1u : 0u);
                }
                tc::commit(bar(B_D1FULL));
                ok = tc::mbar_wait(bar(B_EPI1), (uint32_t)j & 1, &g_fstc_error, E_MMA_WAIT, WAIT_CYCLES);
                if (ok && j > 0)
                    ok = tc::mbar_wait(bar(B_EPI2), (uint32_t)(j - 1) & 1, &g_fstc_error, E_MMA_WAIT, WAIT_CYCLES);
                if (!ok) break;
                tc::fence_after();
#pragma unroll
                for (int t = 0; t < 4; t++) {
#pragma unroll
                    for (int kk = 0; kk < 4; kk++) {
                        const uint64_t da = tc::smem_desc(sbase + OFF_A2 + t * A2_TILE + 32u * kk, 16, 1024, tc::SW128);
                        const uint64_t db = tc::smem_desc(sbase + OFF_B2 + 32u * kk, 16, 1024, tc::SW128);
                        tc::mma_f16(tmem + 256u + 32u * t, da, db, id2, kk ? 1u : 0u);
                    }
                }
                tc::commit(bar(B_D2FULL));
            }
            // completes once every MMA issued above has finished
            tc::commit(bar(B_DRAIN));
            tc::mbar_wait(bar(B_DRAIN), 0, &g_fstc_error, E_MMA_WAIT, WAIT_CYCLES);
        }
        __syncwarp();
    } else if (warp == 9) {
        // ------------------------------ store warp ------------------------------
        // Unit j's spectra, repacked by the workers into sample buffer j & 1
        // as [2C][G] FP16 rows, go out as TMA stores (3D boxes of 256 output
        // rows); STORED completes once the buffer has been read.
        if (lane == 0) {
            for (int j = 0; j < nunits; j++) {
                if (!tc::mbar_wait(bar(B_REPACK), (uint32_t)j & 1, &g_fstc_error, E_STORE_WAIT, WAIT_CYCLES)) break;
                const uint32_t u = blockIdx.x + (uint32_t)j * gridDim.x;      // 32-bit: no FP64-assisted division
                const int s = (int)(u / (uint32_t)args.units_k), k0 = (int)(u % (uint32_t)args.units_k) * G;
                const uint32_t src = sbase + OFF_B1 + (uint32_t)(j & 1) * B1_BYTES;
#pragma unroll 1
                for (int b = 0; b < (FC * 2) / 256; b++) tma_store_3d(src + 4096u * b, &tmap_out, k0, s, 256 * b);
                bulk_commit();
                bulk_wait_read();
                tc::mbar_arrive(bar(B_STORED));
            }
            bulk_wait_all();
        }
        __syncwarp();
    } else {
        // ------------------------------ workers ------------------------------
        const int q = warp & 3, h = warp >> 2;        // TMEM lane quarter, segment half
        const int64_t chunks = a.bytes_per_input >> 4;

        // twiddles W_2048^(n2 k1) of this thread's epilogue-1 values:
        // k1 = 16 q + 8 gi + lane/4, n2 = 8 m + 2 (lane%4) + e
        float2 tw[2][4][2];
#pragma unroll
        for (int gi = 0; gi < 2; gi++)
#pragma unroll
            for (int m = 0; m < 4; m++)
#pragma unroll
                for (int e = 0; e < 2; e++) {
                    const int k1 = 16 * q + 8 * gi + (lane >> 2), n2 = 8 * m + 2 * (lane & 3) + e;
                    float sn, cs;
                    sincospif(-(float)((n2 * k1) & 2047) / 1024.0f, &sn, &cs);
                    tw[gi][m][e] = make_float2(cs, sn);
                }

        auto unit_of = [&](int j, int& s, int& k0) {
            const uint32_t u = blockIdx.x + (uint32_t)j * gridDim.x;
            s = (int)(u / (uint32_t)args.units_k);
            k0 = (int)(u % (uint32_t)args.units_k) * G;
        };
        // raw chunks of unit j -> raw buffer j & 1 (zero outside the input)
        auto fetch = [&](int j) {
            int s, k0;
            unit_of(j, s, k0);
            const unsigned char* base = a.raw + (int64_t)s * a.bytes_per_input;
            const uint32_t dst0 = sbase + OFF_RAW + (uint32_t)(j & 1) * RAW_BYTES;
            for (int i = tid; i < G * RAWC; i += WORKERS) {
                const int g = i / RAWC, c = i % RAWC, k = k0 + g;
                const bool kv = k < K;
                const int64_t start = a.start_sample + (int64_t)k * FN +
                                      ((a.shift && kv) ? __ldg(a.shift + (int64_t)s * K + k) : 0);
                const int64_t ci = (start >> 6) + c;
                const bool ok = kv && ci >= 0 && ci < chunks;
                cp_async16(dst0 + 16u * i, ok ? base + 16 * ci : a.raw, ok);
                if (c == 0) offs[(j & 1) * G + g] = (int)(start & 63);
            }
            cp_async_commit();
        };
        // unpack unit j (raw buffer j & 1) -> B1 buffer j & 1:
        // element (n1, 32 g + n2) = sample 32 n1 + n2 of segment g
        auto decode = [&](int j) {
            const uint32_t* rw0 = reinterpret_cast<const uint32_t*>(sm + OFF_RAW + (j & 1) * RAW_BYTES);
            unsigned char* b1 = sm + OFF_B1 + (j & 1) * B1_BYTES;
#pragma unroll
            for (int r = 0; r < 4; r++) {
                const int idx = tid + WORKERS * r;
                const int g = idx >> 7, wd = idx & 127;
                const int off = offs[(j & 1) * G + g];
                const uint32_t* rw = rw0 + g * RAWC * 4 + (off >> 4) + wd;
                const uint32_t bits = __funnelshift_r(rw[0], rw[1], 2 * (off & 15));
                uint32_t hv[8];
#pragma unroll
                for (int p = 0; p < 8; p++) {
                    const __half2 v = lut2[(bits >> (4 * p)) & 15u];
                    hv[p] = *reinterpret_cast<const uint32_t*>(&v);
                }
                const int n1 = wd >> 1;
                const int chunk = 4 * (g & 1) + 2 * (wd & 1);
                unsigned char* rowp = b1 + (g >> 1) * 8192 + n1 * 128;
                *reinterpret_cast<uint4*>(rowp + (((chunk ^ n1) & 7) << 4)) = make_uint4(hv[0], hv[1], hv[2], hv[3]);
                *reinterpret_cast<uint4*>(rowp + ((((chunk + 1) ^ n1) & 7) << 4)) = make_uint4(hv[4], hv[5], hv[6], hv[7]);
            }
        };

        // Order per unit j: epilogue 1 (j), unpack (j+1) while pass 2 of j
        // runs, epilogue 2 and write-out (j) while pass 1 of j+1 runs.  Raw
        // words run two units ahead: unit j+2 is fetched into the raw buffer
        // unit j used once unit j+1 is unpacked.
        bool ok = true;
        if (nunits > 0) {
            fetch(0);
            if (nunits > 1) fetch(1);
            cp_async_wait_all();
            worker_bar();
            decode(0);
            tc::fence_proxy_async();
            tc::mbar_arrive(bar(B_B1FULL0));
        }
        for (int j = 0; j < nunits; j++) {
            int s, k0;
            unit_of(j, s, k0);

            // ---- epilogue 1: Y -> Z = Y W_2048^(n2 k1) -> A2 (FP16) ----
            ok = tc::mbar_wait(bar(B_D1FULL), (uint32_t)j & 1, &g_fstc_error, E_WORKER_WAIT, WAIT_CYCLES);
            if (!worker_vote(ok)) { ok = false; break; }
            tc::fence_after();
            {
                // the next segment's TMEM loads are in flight while this one is
                // twiddled and stored
                uint32_t rr[2][2][16];
                auto load = [&](int sg, uint32_t (&dst)[2][16]) {
                    const uint32_t col = 32u * (uint32_t)(4 * h + sg);
                    tc::tmem_ld_16x256b_x4(tmem + ((uint32_t)(32 * q) << 16) + col, dst[0]);
                    tc::tmem_ld_16x256b_x4(tmem + ((uint32_t)(32 * q + 16) << 16) + col, dst[1]);
                };
                load(0, rr[0]);
                tc::tmem_ld_wait();
                pin16(rr[0][0]);
                pin16(rr[0][1]);
#pragma unroll
                for (int sg = 0; sg < 4; sg++) {
                    if (sg < 3) load(sg + 1, rr[(sg + 1) & 1]);
                    const int g = 4 * h + sg;                  // segment in the unit
                    unsigned char* tile = sm + OFF_A2 + (g >> 1) * A2_TILE;
#pragma unroll
                    for (int gi = 0; gi < 2; gi++) {
                        const uint32_t (&r)[16] = rr[sg & 1][gi];
                        const int k1 = 16 * q + 8 * gi + (lane >> 2);
                        const uint32_t row = 64 * (g & 1) + k1;
#pragma unroll
                        for (int m = 0; m < 4; m++) {
                            const float2 y0 = make_float2(__uint_as_float(r[4 * m]), __uint_as_float(r[4 * m + 2]));
                            const float2 y1 = make_float2(__uint_as_float(r[4 * m + 1]), __uint_as_float(r[4 * m + 3]));
                            const float2 z0 = cmul(y0, tw[gi][m][0]), z1 = cmul(y1, tw[gi][m][1]);
                            const __half2 re = __floats2half2_rn(z0.x, z1.x), im = __floats2half2_rn(z0.y, z1.y);
                            const uint32_t kpos = 8 * m + 2 * (lane & 3);
                            *reinterpret_cast<__half2*>(tile + sw128(row, kpos)) = re;
                            *reinterpret_cast<__half2*>(tile + sw128(row, 32 + kpos)) = im;
                        }
                    }
                    if (sg < 3) {
                        tc::tmem_ld_wait();
                        pin16(rr[(sg + 1) & 1][0]);
                        pin16(rr[(sg + 1) & 1][1]);
                    }
                }
            }
            tc::fence_before();
            tc::fence_proxy_async();
            tc::mbar_arrive(bar(B_EPI1));

            if (j + 1 < nunits) {
                // sample buffer (j+1) & 1 held unit j-1's spectra for the store warp
                ok = j == 0 || tc::mbar_wait(bar(B_STORED), (uint32_t)(j - 1) & 1, &g_fstc_error, E_WORKER_WAIT,
                                             WAIT_CYCLES);
                if (!worker_vote(ok)) { ok = false; break; }
                cp_async_wait_all();
                worker_bar();                                   // every thread's copies have landed,
                decode(j + 1);                                  // and unit j's raw buffer is released
                tc::fence_proxy_async();
                tc::mbar_arrive(bar((j + 1) & 1));
            }
            if (j + 2 < nunits) fetch(j + 2);

            // ---- epilogue 2: X -> phasor, scale -> FP16 staging ----
            ok = tc::mbar_wait(bar(B_D2FULL), (uint32_t)j & 1, &g_fstc_error, E_WORKER_WAIT, WAIT_CYCLES);
            if (!worker_vote(ok)) { ok = false; break; }          // (also: staging is free again)
            tc::fence_after();
            __half2* stg = reinterpret_cast<__half2*>(sm + OFF_STG);
            {
                const int k1 = 32 * (q & 1) + lane;
                uint32_t re[2][16], im[2][16];
#pragma unroll
                for (int tt = 0; tt < 2; tt++) {
                    const uint32_t ta = tmem + ((uint32_t)(32 * q) << 16) + 256u + 32u * (uint32_t)(2 * h + tt);
                    tc::tmem_ld_32x32b_x16(ta, re[tt]);
                    tc::tmem_ld_32x32b_x16(ta + 16, im[tt]);
                }
                tc::tmem_ld_wait();
#pragma unroll
                for (int tt = 0; tt < 2; tt++) {
                    pin16(re[tt]);
                    pin16(im[tt]);
                }
                const float* scl = a.scale ? a.scale + (int64_t)s * FC : nullptr;
#pragma unroll
                for (int tt = 0; tt < 2; tt++) {
                    const int g = 2 * (2 * h + tt) + (q >> 1);   // segment of this TMEM lane quarter
                    float2 B = make_float2(1.f, 0.f), D = B;
                    if (PHASE) {
                        const int64_t sk = (int64_t)s * K + k0 + g;
                        const float ph0 = __ldg(a.phase0 + sk), dph = __ldg(a.dphase + sk);
                        float sn, cs;
                        sincosf(ph0 + (float)k1 * dph, &sn, &cs);
                        B = make_float2(cs, sn);
                        sincosf(64.f * dph, &sn, &cs);
                        D = make_float2(cs, sn);
                    }
#pragma unroll
                    for (int k2 = 0; k2 < 16; k2++) {
                        float2 X = make_float2(__uint_as_float(re[tt][k2]), __uint_as_float(im[tt][k2]));
                        const int c = k1 + 64 * k2;
                        if (PHASE) {
                            X = cmul(X, B);
                            B = cmul(B, D);
                        }
                        if (scl) X = cscale(X, __ldg(scl + c));
                        stg[c * (G + 1) + g] = __floats2half2_rn(X.x, X.y);
                    }
                }
            }
            tc::fence_before();
            tc::mbar_arrive(bar(B_EPI2));
            worker_bar();

            // ---- corner-turned write-out of the unit's G segments ----
            // Row r = 2c + plane of the output ([C][2][S][kp] FP16) gets the G
            // halves k0..k0+7 of input s: repacked as [2C][G] into sample
            // buffer j & 1 (pass 1 of unit j is done with it) for the store warp.
            {
                uint4* rows = reinterpret_cast<uint4*>(sm + OFF_B1 + (j & 1) * B1_BYTES);
                for (int idx = tid; idx < FC * 2; idx += WORKERS) {
                    const int plane = idx & 1, c = idx >> 1;
                    const uint32_t* w = reinterpret_cast<const uint32_t*>(stg + c * (G + 1));
                    const uint32_t sel = plane ? 0x7632u : 0x5410u;
                    rows[idx] = make_uint4(__byte_perm(w[0], w[1], sel), __byte_perm(w[2], w[3], sel),
                                           __byte_perm(w[4], w[5], sel), __byte_perm(w[6], w[7], sel));
                }
                tc::fence_proxy_async();
                tc::mbar_arrive(bar(B_REPACK));
            }
        }
        cp_async_wait_all();
        tc::fence_before();
    }
    __syncthreads();
    if (warp == 8) {
        tc::fence_after();
        tc::tmem_dealloc(tmem, TMEM_COLS);
    }
}

// A1 (DFT-64, rows ordered Re/Im per 8 k1) and B2 (DFT-32 as a real 32 x 64
// operand) in FP16, 128-byte-swizzled K-major, one copy per device.
std::mutex g_const_mu;
std::map<int, uint4*> g_consts;

const uint4* tc_constants()
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
        const int k1 = 8 * (r / 16) + (r % 8), part = (r % 16) / 8;
        for (int n1 = 0; n1 < 64; n1++) {
            const double th = 2.0 * M_PI * (double)((n1 * k1) % 64) / 64.0;
            put(OFF_A1, r, n1, part == 0 ? std::cos(th) : -std::sin(th));
        }
    }
    for (int r = 0; r < 32; r++) {
        const int k2 = r % 16, part = r / 16;
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

int g_sms = 0;

}  // namespace

bool cs_fstage_tc_supported(const CsFStageArgs& a)
{
    // K % 8: whole units of 8 segments and a 16-byte TMA row pitch
    return a.N == FN && a.format == CS_SPECTRA_F16 && !a.msb_first && a.K % G == 0;
}

int cs_fx_fstage_tc(const CsFStageArgs& a, cudaStream_t st)
{
    if (!cs_fstage_tc_supported(a)) return CS_ERR_UNSUPPORTED;
    if ((int64_t)a.S * ((a.K + G - 1) / G) >= (int64_t)1 << 31) return CS_ERR_UNSUPPORTED;   // 32-bit unit indices
    if (!a.raw || !a.out || a.S <= 0 || a.K <= 0) return CS_ERR_ARG;
    if ((uintptr_t)a.raw % 16 || a.bytes_per_input % 16 || (uintptr_t)a.out % 16) return CS_ERR_ARG;
    const uint4* consts = tc_constants();
    if (!consts) return (int)cudaErrorMemoryAllocation;
    if (!g_sms) {
        int dev = 0, n = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        g_sms = n > 0 ? n : 148;
    }
    const CsEncodeTiledFn enc = cs_encode_tiled();
    if (!enc) return CS_ERR_UNSUPPORTED;
    // output as a 3D FP16 tensor: x = segment (K), y = input (S), z = 2c + plane
    CUtensorMap tm;
    const cuuint64_t gdim[3] = {(cuuint64_t)a.K, (cuuint64_t)a.S, (cuuint64_t)FC * 2};
    const int kp = a.kp ? a.kp : a.K;
    if (kp < a.K || kp % 8) return CS_ERR_ARG;
    const int s_rows = a.S_out ? a.S_out : a.S;
    const cuuint64_t gstride[2] = {(cuuint64_t)kp * 2, (cuuint64_t)kp * s_rows * 2};
    const cuuint32_t box[3] = {G, 1, 256};
    const cuuint32_t estr[3] = {1, 1, 1};
    if (enc(&tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 3, a.out, gdim, gstride, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) !=
        CUDA_SUCCESS)
        return CS_ERR_ARG;
    void* errp = nullptr;
    CS_CUDA_TRY(cudaGetSymbolAddress(&errp, g_fstc_error));
    CS_CUDA_TRY(cudaMemsetAsync(errp, 0, sizeof(unsigned), st));
    TcFArgs t{};
    t.f = a;
    t.consts = consts;
    t.units_k = (a.K + G - 1) / G;
    t.units = (int64_t)a.S * t.units_k;
    const int grid = (int)std::min<int64_t>(t.units, g_sms);
    if (a.phase0) {
        CS_CUDA_TRY(cs_smem_at_least(reinterpret_cast<const void*>(k_fx_fstage_tc<true>), (int)(SMEM_BYTES)));
        k_fx_fstage_tc<true><<<grid, THREADS, SMEM_BYTES, st>>>(t, tm), cs_count_launches(1);
    } else {
        CS_CUDA_TRY(cs_smem_at_least(reinterpret_cast<const void*>(k_fx_fstage_tc<false>), (int)(SMEM_BYTES)));
        k_fx_fstage_tc<false><<<grid, THREADS, SMEM_BYTES, st>>>(t, tm), cs_count_launches(1);
    }
    return (int)cudaGetLastError();
}

int cs_fstage_tc_status(unsigned* code)
{
    return (int)cudaMemcpyFromSymbol(code, g_fstc_error, sizeof(unsigned));
}
