// K-d2, INT8 form: the X stage on int8 spectra with int32 accumulation.
//
// tcgen05 has no kind::i8 on sm_103a (ptxas: "Feature '.kind::i8' not
// supported on .target 'sm_103a'"), so on GB300 the only INT8 tensor path is
// the warp-level mma.sync IMMA (m16n8k32, s8 x s8 -> s32).  This file is that
// X stage, built to measure what INT8 gives against the tcgen05 FP16 one:
//
//  * k_quantise_i8: per (channel, input) row of FP32 spectra the largest |Re|
//    or |Im| sets the scale s = max / 127; Re and Im become int8 rows
//    rint(x / s) of planes [C][2][S][kp] and scale[s][c] = s.
//  * k_xmac_i8: one CTA per 128 x 128 (i, j) tile touching the lower triangle
//    of one channel, 16 warps of 32 x 32; operands K-major in shared memory
//    (80-byte rows: conflict-free ldmatrix), a 4-stage cp.async ring of
//    64-byte k-chunks; per k32 step and 16 x 8 block four IMMAs
//        Re += Ar Br^T + Ai Bi^T,   Im += Ai Br^T + Ar (-Bi)^T
//    (-Bi negated bytewise in registers; quantised values are within +-127);
//    epilogue V_ij = s_i s_j (Re + i Im) in FP32, the conjugate MAC of
//    genericAddProduct_32fc_conj (architecture.h:427-433) for every product.
#include "common.cuh"
#include "kernels.h"

#include <cuda_runtime.h>

#include <mutex>
#include <vector>

namespace {

constexpr int TM = 128, TN = 128, KCH = 64;      // tile and k-chunk (bytes = int8 elements)
constexpr int ROW = 80;                          // shared row pitch: 64 bytes + 16 (bank spread)
constexpr int NST = 4;                           // pipeline stages
constexpr int WARPS = 16, THREADS = WARPS * 32;
constexpr int OP_BYTES = TM * ROW;               // one operand tile (Ar, Ai, Br or Bi)
constexpr int STAGE = 4 * OP_BYTES;
constexpr int SMEM = NST * STAGE;                // 160 KB

CS_DEV uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

CS_DEV void cp16(uint32_t dst, const void* src, bool ok)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(ok ? 16 : 0) : "memory");
}

CS_DEV void ldsm_x4(uint32_t addr, uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3)
{
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(addr));
}

CS_DEV void imma(int (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1)
{
    asm volatile("mma.sync.aligned.m16n8k32.row.col.s32.s8.s8.s32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                 "{%0,%1,%2,%3};"
                 : "+r"(d[0]), "+r"(d[1]), "+r"(d[2]), "+r"(d[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

struct I8Args {
    const int8_t* planes;       // [C][2][S][kp]
    int S, C, K, kp;
    int64_t P;
    const int2* tiles;
    float2* vis;                // [C][P]
    const float* scale;         // [S][stride]
    int stride;
    int accumulate;
};

__global__ void __launch_bounds__(THREADS, 1) k_xmac_i8(const I8Args a)
{
    extern __shared__ __align__(128) unsigned char sm[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int2 tile = a.tiles[blockIdx.x];
    const int c = blockIdx.y, i0 = tile.x, j0 = tile.y, S = a.S;
    const int nk = (a.K + KCH - 1) / KCH;
    const int8_t* re_rows = a.planes + (int64_t)(c * 2 + 0) * S * a.kp;
    const int8_t* im_rows = a.planes + (int64_t)(c * 2 + 1) * S * a.kp;

    // stage fill: 4 operands x 128 rows x 4 pieces of 16 bytes = 2048 pieces, 4 per thread
    auto fill = [&](int kc, int slot) {
        const uint32_t base = smem_addr(sm + slot * STAGE);
#pragma unroll
        for (int t = 0; t < 4; t++) {
            const int piece = threadIdx.x + t * THREADS;
            const int op = piece >> 9, r = (piece >> 2) & 127, q = piece & 3;
            const int row = (op < 2 ? i0 : j0) + r;
            const int k = kc * KCH + 16 * q;
            const bool ok = row < S && k < a.K;
            const int8_t* src = (op & 1) ? im_rows : re_rows;
            cp16(base + op * OP_BYTES + r * ROW + 16 * q, ok ? src + (int64_t)row * a.kp + k : a.planes, ok);
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    };

    const int wi = warp >> 2, wj = warp & 3;         // warp tile: rows 32 wi.., columns 32 wj..
    int accr[2][4][4], acci[2][4][4];
#pragma unroll
    for (int m = 0; m < 2; m++)
#pragma unroll
        for (int n = 0; n < 4; n++)
#pragma unroll
            for (int e = 0; e < 4; e++) accr[m][n][e] = acci[m][n][e] = 0;

    for (int s = 0; s < NST - 1; s++) {
        if (s < nk) fill(s, s);
        else asm volatile("cp.async.commit_group;" ::: "memory");
    }
    // ldmatrix lanes: matrices (rows 0-7 | 8-15) x (k 0-15 | 16-31) of an m16 x k32 block
    const int lr = lane & 15, lk = (lane >> 4) * 16;
    for (int kc = 0; kc < nk; kc++) {
        asm volatile("cp.async.wait_group %0;" ::"n"(NST - 2) : "memory");
        __syncthreads();
        // the slot freed by the previous iteration takes chunk kc + NST - 1
        if (kc + NST - 1 < nk) fill(kc + NST - 1, (kc + NST - 1) % NST);
        else asm volatile("cp.async.commit_group;" ::: "memory");
        const uint32_t st = smem_addr(sm + (kc % NST) * STAGE);
#pragma unroll
        for (int ks = 0; ks < 2; ks++) {
            uint32_t ar[2][4], ai[2][4], br[4][2], bi[4][2];
#pragma unroll
            for (int m = 0; m < 2; m++) {
                const uint32_t off = (uint32_t)((32 * wi + 16 * m + lr) * ROW + 32 * ks + lk);
                ldsm_x4(st + 0 * OP_BYTES + off, ar[m][0], ar[m][1], ar[m][2], ar[m][3]);
                ldsm_x4(st + 1 * OP_BYTES + off, ai[m][0], ai[m][1], ai[m][2], ai[m][3]);
            }
            // B: matrices (n rows 0-7, k 0-15), (same, k 16-31), (n rows 8-15, k 0-15), (.., k 16-31)
#pragma unroll
            for (int n2 = 0; n2 < 2; n2++) {
                const int nrow = 32 * wj + 16 * n2 + (lane & 7) + ((lane >> 4) << 3);
                const uint32_t off = (uint32_t)(nrow * ROW + 32 * ks + ((lane >> 3) & 1) * 16);
                ldsm_x4(st + 2 * OP_BYTES + off, br[2 * n2][0], br[2 * n2][1], br[2 * n2 + 1][0], br[2 * n2 + 1][1]);
                ldsm_x4(st + 3 * OP_BYTES + off, bi[2 * n2][0], bi[2 * n2][1], bi[2 * n2 + 1][0], bi[2 * n2 + 1][1]);
            }
#pragma unroll
            for (int n = 0; n < 4; n++) {
                const uint32_t nb0 = __vneg4(bi[n][0]), nb1 = __vneg4(bi[n][1]);
#pragma unroll
                for (int m = 0; m < 2; m++) {
                    imma(accr[m][n], ar[m], br[n][0], br[n][1]);
                    imma(accr[m][n], ai[m], bi[n][0], bi[n][1]);
                    imma(acci[m][n], ai[m], br[n][0], br[n][1]);
                    imma(acci[m][n], ar[m], nb0, nb1);
                }
            }
        }
    }
    asm volatile("cp.async.wait_group 0;" ::: "memory");

    // epilogue: thread holds rows g, g + 8 and columns 2 t, 2 t + 1 of each 16 x 8 block
    const int g = lane >> 2, t4 = lane & 3;
#pragma unroll
    for (int m = 0; m < 2; m++)
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int i = i0 + 32 * wi + 16 * m + g + 8 * h;
            if (i >= S) continue;
            const float si = a.scale[(int64_t)i * a.stride + c];
            float2* row = a.vis + (int64_t)c * a.P + (int64_t)i * (i + 1) / 2;
#pragma unroll
            for (int n = 0; n < 4; n++)
#pragma unroll
                for (int e = 0; e < 2; e++) {
                    const int j = j0 + 32 * wj + 8 * n + 2 * t4 + e;
                    if (j > i) continue;
                    const float f = si * a.scale[(int64_t)j * a.stride + c];
                    float2 v = make_float2((float)accr[m][n][2 * h + e] * f, (float)acci[m][n][2 * h + e] * f);
                    if (a.accumulate) {
                        const float2 o = row[j];
                        v.x += o.x;
                        v.y += o.y;
                    }
                    row[j] = v;
                }
        }
}

// One warp per (channel, input) row of FP32 spectra [C][S][kp].
__global__ void k_quantise_i8(const float2* __restrict__ spectra, int S, int C, int K, int kp,
                              int8_t* __restrict__ out, float* __restrict__ scale)
{
    const int64_t row = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (row >= (int64_t)C * S) return;
    const int c = (int)(row / S), s = (int)(row - (int64_t)c * S);
    const float4* x = reinterpret_cast<const float4*>(spectra + row * kp);   // two segments per float4
    float m = 0.f;
    for (int k = 2 * lane; k < K; k += 64) {
        const float4 v = x[k >> 1];
        m = fmaxf(m, fmaxf(fmaxf(fabsf(v.x), fabsf(v.y)), fmaxf(fabsf(v.z), fabsf(v.w))));
    }
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    const float sc = m > 0.f ? m / 127.f : 1.f;
    const float inv = 1.f / sc;
    if (lane == 0) scale[(int64_t)s * C + c] = sc;
    int8_t* re = out + ((int64_t)(c * 2 + 0) * S + s) * kp;
    int8_t* im = out + ((int64_t)(c * 2 + 1) * S + s) * kp;
    auto q = [&](float f) { return (uint32_t)(uint8_t)(int8_t)max(-127, min(127, __float2int_rn(f * inv))); };
    for (int k = 4 * lane; k < K; k += 128) {          // K % 16 == 0: whole groups of 4
        const float4 v0 = x[k >> 1], v1 = x[(k >> 1) + 1];
        *reinterpret_cast<uint32_t*>(re + k) = q(v0.x) | q(v0.z) << 8 | q(v1.x) << 16 | q(v1.z) << 24;
        *reinterpret_cast<uint32_t*>(im + k) = q(v0.y) | q(v0.w) << 8 | q(v1.y) << 16 | q(v1.w) << 24;
    }
}

std::mutex g_i8_mu;
std::vector<std::pair<std::pair<int, int>, int2*>> g_i8_tiles;   // ((device, S) -> lower-triangle tiles)

const int2* i8_tiles(int S, int* n)
{
    std::vector<int2> h;
    for (int i0 = 0; i0 < S; i0 += TM)
        for (int j0 = 0; j0 <= i0; j0 += TN) h.push_back(make_int2(i0, j0));
    *n = (int)h.size();
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(g_i8_mu);
    for (auto& e : g_i8_tiles)
        if (e.first.first == dev && e.first.second == S) return e.second;
    int2* d = nullptr;
    if (cudaMalloc(&d, sizeof(int2) * h.size()) != cudaSuccess) return nullptr;
    if (cudaMemcpy(d, h.data(), sizeof(int2) * h.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(d);
        return nullptr;
    }
    g_i8_tiles.push_back({{dev, S}, d});
    return d;
}

}  // namespace

int cs_xmac_i8(const int8_t* planes, int S, int C, int K, int kp, float2* vis, const float* scale, int scale_stride,
               int accumulate, cudaStream_t st)
{
    if (!planes || !vis || !scale || S <= 0 || C <= 0 || C > 65535 || K <= 0 || kp < K) return CS_ERR_ARG;
    if (K % 16 || kp % 16 || (uintptr_t)planes % 16) return CS_ERR_ARG;
    if (K > 65536) return CS_ERR_UNSUPPORTED;          // |int32 sums| <= 2 K 127^2
    int ntiles = 0;
    const int2* tiles = i8_tiles(S, &ntiles);
    if (!tiles) return CS_ERR_ARG;
    I8Args a{planes, S, C, K, kp, (int64_t)S * (S + 1) / 2, tiles, vis, scale, scale_stride > 0 ? scale_stride : C,
             accumulate};
    CS_CUDA_TRY(cs_smem_at_least(reinterpret_cast<const void*>(k_xmac_i8), (int)(SMEM)));
    k_xmac_i8<<<dim3(ntiles, C), THREADS, SMEM, st>>>(a), cs_count_launches(1);
    return (int)cudaGetLastError();
}

int cs_quantise_i8(const float2* spectra, int S, int C, int K, int kp, int8_t* planes, float* scale, cudaStream_t st)
{
    if (!spectra || !planes || !scale || S <= 0 || C <= 0 || K <= 0 || K % 16 || kp % 16 || kp < K) return CS_ERR_ARG;
    if ((uintptr_t)spectra % 16 || (uintptr_t)planes % 16) return CS_ERR_ARG;
    const int64_t rows = (int64_t)C * S;
    const int64_t blocks = (rows + 7) / 8;
    if (blocks > 0x7fffffffLL) return CS_ERR_ARG;
    k_quantise_i8<<<(unsigned)blocks, 256, 0, st>>>(spectra, S, C, K, kp, planes, scale), cs_count_launches(1);
    return (int)cudaGetLastError();
}
