// K-d1: X stage, FP32 CUDA cores.
//
// V_c[i][j] = sum_k X_i[c][k] * conj(X_j[c][k]) over the lower triangle
// j <= i (autos on the diagonal), the conjugate-MAC of
// genericAddProduct_32fc_conj (architecture.h:427-433), IPP's cross-pol
// accumulate (TaskCoreIPP.cpp:456-487) and zerocorr.c:601-606, done for all
// S(S+1)/2 products of every channel at once.  Per channel it is a Hermitian
// rank-K update, so it is tiled like a GEMM: a CTA owns a 64x64 block of
// (i, j) for one channel and streams 16 time samples per stage through
// shared memory; each of its 128 threads keeps 4x8 complex accumulators
// (32x32 blocks of 32 threads when S <= 32).
// Only blocks on or below the diagonal are launched.
//
// Layout in:  float2 spectra[C][S][K]   (time innermost)
// Layout out: float2 vis[C][P],  p = i(i+1)/2 + j
#include "common.cuh"
#include "kernels.h"

namespace {
constexpr int XK = 16;      // time samples per stage

__device__ __forceinline__ void tile_coords(int t, int& bi, int& bj)
{
    // t enumerates (bi, bj), bj <= bi, row-major over bi
    int b = (int)((sqrtf(8.f * (float)t + 1.f) - 1.f) * 0.5f);
    while ((b + 1) * (b + 2) / 2 <= t) b++;
    while (b * (b + 1) / 2 > t) b--;
    bi = b;
    bj = t - b * (b + 1) / 2;
}

// Tile edge XT (64, or 32 for S <= 32 so that small arrays do not compute
// three empty quarters of every tile); XT^2/32 threads, each keeping 4 x 8
// complex accumulators: rows ti + TI a, columns tj + TJ b.
template <int XT>
__global__ void __launch_bounds__(XT * XT / 32) k_xmac_f32(const float2* __restrict__ spec, int S, int K, int kp,
                                                          float2* __restrict__ vis, int64_t P, int accumulate)
{
    constexpr int NT = XT * XT / 32, TI = XT / 4, TJ = XT / 8, XLD = XT + 1;
    constexpr int ITER = 2 * XT / NT;                // (row, 8-sample chunk) loads per thread per stage
    __shared__ float2 As[2][XK][XLD];
    __shared__ float2 Bs[2][XK][XLD];
    const int c = blockIdx.y;
    int bi, bj;
    tile_coords(blockIdx.x, bi, bj);
    const int i0 = bi * XT, j0 = bj * XT;
    const int tid = threadIdx.x;
    const int ti = tid / TJ;          // rows ti + TI a
    const int tj = tid % TJ;          // cols tj + TJ b
    const float2* base = spec + (int64_t)c * S * kp;

    float2 ra[ITER][8], rb[ITER][8];
    auto gload = [&](int k0) {
#pragma unroll
        for (int it = 0; it < ITER; it++) {
            const int q = tid + it * NT, lrow = q >> 1, lk = (q & 1) * 8;
            const int ai = i0 + lrow, bjr = j0 + lrow;
            const float2* pa = base + (int64_t)min(ai, S - 1) * kp;
            const float2* pb = base + (int64_t)min(bjr, S - 1) * kp;
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const int k = k0 + lk + u;
                const bool kin = k < K;
                ra[it][u] = (ai < S && kin) ? __ldg(pa + k) : make_float2(0.f, 0.f);
                rb[it][u] = (bjr < S && kin) ? __ldg(pb + k) : make_float2(0.f, 0.f);
            }
        }
    };
    auto sstore = [&](int buf) {
#pragma unroll
        for (int it = 0; it < ITER; it++) {
            const int q = tid + it * NT, lrow = q >> 1, lk = (q & 1) * 8;
#pragma unroll
            for (int u = 0; u < 8; u++) {
                As[buf][lk + u][lrow] = ra[it][u];
                Bs[buf][lk + u][lrow] = rb[it][u];
            }
        }
    };

    float accr[4][8], acci[4][8];
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 8; b++) accr[a][b] = acci[a][b] = 0.f;

    const int nst = (K + XK - 1) / XK;
    gload(0);
    sstore(0);
    __syncthreads();
    for (int stg = 0; stg < nst; stg++) {
        const int cur = stg & 1;
        if (stg + 1 < nst) gload((stg + 1) * XK);
#pragma unroll
        for (int kk = 0; kk < XK; kk++) {
            float2 av[4], bv[8];
#pragma unroll
            for (int a = 0; a < 4; a++) av[a] = As[cur][kk][ti + TI * a];
#pragma unroll
            for (int b = 0; b < 8; b++) bv[b] = Bs[cur][kk][tj + TJ * b];
#pragma unroll
            for (int a = 0; a < 4; a++)
#pragma unroll
                for (int b = 0; b < 8; b++) {
                    accr[a][b] = fmaf(av[a].x, bv[b].x, accr[a][b]);
                    accr[a][b] = fmaf(av[a].y, bv[b].y, accr[a][b]);
                    acci[a][b] = fmaf(av[a].y, bv[b].x, acci[a][b]);
                    acci[a][b] = fmaf(-av[a].x, bv[b].y, acci[a][b]);
                }
        }
        if (stg + 1 < nst) sstore(cur ^ 1);
        __syncthreads();
    }

    float2* out = vis + (int64_t)c * P;
#pragma unroll
    for (int a = 0; a < 4; a++) {
        int i = i0 + ti + TI * a;
        if (i >= S) continue;
#pragma unroll
        for (int b = 0; b < 8; b++) {
            int j = j0 + tj + TJ * b;
            if (j > i) continue;
            int64_t p = (int64_t)i * (i + 1) / 2 + j;
            float2 v = make_float2(accr[a][b], acci[a][b]);
            if (accumulate) {
                float2 o = out[p];
                v.x += o.x;
                v.y += o.y;
            }
            out[p] = v;
        }
    }
}

__global__ void k_vis_transpose(const float2* __restrict__ in, float2* __restrict__ out, int C, int64_t P)
{
    __shared__ float2 tile[32][33];
    int64_t p0 = (int64_t)blockIdx.x * 32;
    int c0 = blockIdx.y * 32;
    int tx = threadIdx.x, ty = threadIdx.y;
    for (int r = ty; r < 32; r += 8) {
        int c = c0 + r;
        int64_t p = p0 + tx;
        if (c < C && p < P) tile[r][tx] = in[(int64_t)c * P + p];
    }
    __syncthreads();
    for (int r = ty; r < 32; r += 8) {
        int64_t p = p0 + r;
        int c = c0 + tx;
        if (c < C && p < P) out[p * C + c] = tile[tx][r];
    }
}
}  // namespace

int cs_xmac_f32(const float2* spectra, int S, int C, int K, int kp, float2* vis, int accumulate, cudaStream_t st)
{
    if (!spectra || !vis || S <= 0 || C <= 0 || K <= 0 || kp < K) return CS_ERR_ARG;
    if (C > 65535) return CS_ERR_ARG;
    const int xt = S <= 32 ? 32 : 64;
    int nb = (S + xt - 1) / xt;
    int64_t tiles = (int64_t)nb * (nb + 1) / 2;
    int64_t P = (int64_t)S * (S + 1) / 2;
    dim3 grid((unsigned)tiles, C);
    if (xt == 32)
        k_xmac_f32<32><<<grid, 32, 0, st>>>(spectra, S, K, kp, vis, P, accumulate);
    else
        k_xmac_f32<64><<<grid, 128, 0, st>>>(spectra, S, K, kp, vis, P, accumulate);
    cs_count_launches(1);
    return (int)cudaGetLastError();
}

int cs_vis_to_baseline_major(const float2* vis_cp, float2* vis_pc, int C, int64_t P, cudaStream_t st)
{
    if (!vis_cp || !vis_pc || C <= 0 || P <= 0) return CS_ERR_ARG;
    dim3 grid((unsigned)((P + 31) / 32), (C + 31) / 32);
    k_vis_transpose<<<grid, dim3(32, 8), 0, st>>>(vis_cp, vis_pc, C, P), cs_count_launches(1);
    return (int)cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Batched service jobs: several small jobs' inputs run as one stacked job;
// each job's products are gathered from the stacked channel-major triangle.
// ---------------------------------------------------------------------------
namespace {

__global__ void k_vis_gather(const __grid_constant__ CsGatherArgs a)
{
    const CsGatherJob& J = a.job[blockIdx.y];
    const int64_t P = (int64_t)J.S * (J.S + 1) / 2, total = (int64_t)a.C * P;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        int64_t c, p;
        if (J.baseline_major) p = t / a.C, c = t - p * a.C;
        else c = t / P, p = t - c * P;
        // p = i (i + 1) / 2 + j, j <= i: i from the root, corrected by one step either way
        int i = (int)((sqrtf(8.f * (float)p + 1.f) - 1.f) * 0.5f);
        while ((int64_t)i * (i + 1) / 2 > p) i--;
        while ((int64_t)(i + 1) * (i + 2) / 2 <= p) i++;
        const int j = (int)(p - (int64_t)i * (i + 1) / 2);
        const int64_t gi = J.off + i, gj = J.off + j;
        const float2 v = a.src[c * a.P_stacked + gi * (gi + 1) / 2 + gj];
        J.dst[J.baseline_major ? p * a.C + c : c * P + p] = v;
    }
}

}  // namespace

int cs_vis_gather(const CsGatherArgs& a, cudaStream_t st)
{
    if (!a.src || a.n <= 0 || a.n > CS_GATHER_MAX || a.C <= 0) return CS_ERR_ARG;
    k_vis_gather<<<dim3(152, a.n), 256, 0, st>>>(a), cs_count_launches(1);
    return (int)cudaGetLastError();
}
