// K-d2: X stage on the tcgen05 tensor cores (FP16 operands, FP32 accumulate).
//
// Per channel c the visibilities are the Hermitian rank-K product V = X X^H
// of the S x K spectra matrix X = Xr + i Xi (the conjugate MAC of
// genericAddProduct_32fc_conj, architecture.h:427-433, for every product):
//     Re V = Xr Xr^T + Xi Xi^T,      Im V = Xi Xr^T - Xr Xi^T.
// A CTA owns one 128 (i) x 128 (j) tile of one channel that touches the lower
// triangle.  Its two FP32 accumulators live in tensor memory (TMEM): columns
// 0..127 hold Re V, 128..255 hold Im V, lane = row i, so two CTAs share an
// SM's TMEM and one's epilogue overlaps the other's MMAs.  Each k-step issues
// four kind::f16 MMAs (M=128, N=128, K=16); the minus sign of the last product
// is the instruction descriptor's negate-A bit, so no negated copy of the data
// exists.  Operands are K-major (time innermost), loaded by TMA with 64-byte
// swizzle into a 3-stage shared-memory ring (32 KB stages) guarded by
// mbarriers.  A diagonal tile (i0 = j0) loads its rows once and uses them as
// both operands, and needs three MMAs per k-step: its Im columns accumulate
// M = Xi Xr^T and the epilogue forms Im V = M - M^T through shared memory.
//
// Warp roles (6 warps): warp 0 = TMA producer, warp 1 = TMEM owner and MMA
// issuer, warps 2..5 = epilogue (TMEM -> registers -> global; warp w reads
// TMEM lanes 32*(w%4)..+31).  Every mbarrier wait is bounded: on timeout the
// kernel records an error code, drains its own copies (bounded), frees TMEM
// and returns, and the host reports the failure.
//
// Layout in:  __half spectra[C][2][S][K]  (plane 0 = Re, plane 1 = Im), or
//             k-blocked [C][S][K/32][2][32] (4-D tensor map), or channel-grouped
//             k-blocked [C/16][S][K/32][16][2][32] (5-D tensor map)
// Layout out: float2 vis[C][P], p = i(i+1)/2 + j, j <= i
#include <cuda.h>

#include "common.cuh"
#include "kernels.h"
#include "tcgen05.cuh"
#include "tma.h"

#include <mutex>
#include <vector>

namespace {

constexpr int BM = 128, BN = 128, BK = 32;          // tile and k-chunk (64 B of FP16 = one swizzle row)
constexpr int STAGES = 3;
constexpr int A_BYTES = BM * BK * 2;                // 8 KB
constexpr int B_BYTES = BN * BK * 2;                // 8 KB
constexpr int STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;   // Ar, Ai, Br, Bi = 32 KB
constexpr int TC_THREADS = 192;
// epilogue shared memory: four warps' 32 x 17 float2 staging blocks, then (on
// a diagonal tile) M as [BM][MP] floats; both inside the operand ring
constexpr int EPI_STG_BYTES = 4 * 32 * 17 * 8;
constexpr int MP = BM + 1;
static_assert(EPI_STG_BYTES + BM * MP * 4 <= STAGES * STAGE_BYTES, "epilogue M staging inside the ring");
constexpr uint32_t TMEM_COLS = 256;
constexpr long long WAIT_CYCLES = 4000000000LL;     // ~2 s at 2 GHz

// error codes written to g_tc_error
constexpr unsigned ERR_FULL_WAIT = 1, ERR_EMPTY_WAIT = 2, ERR_ACC_WAIT = 3;

__device__ unsigned g_tc_error;

using tc::smem_u32;

// Bounded wait: false (and the error code recorded in g_tc_error) after WAIT_CYCLES.
CS_DEV bool mbar_wait(uint32_t bar, uint32_t parity, unsigned code)
{
    return tc::mbar_wait(bar, parity, &g_tc_error, code, WAIT_CYCLES);
}

// K-major operand in shared memory with 64-byte swizzle: 8-row x 64-byte
// atoms stacked along M/N every 512 bytes (stride byte offset).
CS_DEV uint64_t sw64_desc(uint32_t saddr) { return tc::smem_desc(saddr, 16, 512, tc::SW64); }

// the four epilogue warps (2..5): named barrier 1 over their 128 threads, and
// an AND vote on it that every one of them reaches
CS_DEV void epi_bar() { asm volatile("bar.sync 1, 128;" ::: "memory"); }
CS_DEV bool epi_vote(bool ok)
{
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "bar.red.and.pred q, 1, 128, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(r)
        : "r"(ok ? 1u : 0u)
        : "memory");
    return r != 0;
}

struct TcArgs {
    int S, C, K;
    int64_t P;
    const int2* tiles;          // (i0, j0) per tile
    float2* vis;
    const float* inv_scale;     // [S][scale_stride] or null
    int scale_stride;
    int accumulate;
    int box_rows;               // rows per TMA box: BM, or S rounded up to 8 when S < BM
    int small;                  // S <= BM: one tile per channel whose B operand is its A operand
    uint32_t tmem_cols;         // TMEM columns: Re V in [0, cols/2), Im V in [cols/2, cols)
    int kblock;                 // spectra k-blocked: 1 [C][S][kp/32][2][32] (4-D tensor map),
                                // 2 channel-grouped [C/16][S][kp/32][16][2][32] (5-D)
};

__global__ void __launch_bounds__(TC_THREADS, 1) k_xmac_tc(const __grid_constant__ CUtensorMap tmap,
                                                           const __grid_constant__ TcArgs a)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    // offset from the shared array itself (not an integer round trip), so that
    // the compiler keeps shared-space 32-bit addressing for every access
    unsigned char* smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
    // S <= BM: a stage holds Ar and Ai only (the tile is diagonal, B = A)
    const uint32_t stage_bytes = a.small ? 2 * A_BYTES : STAGE_BYTES;
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + STAGES * stage_bytes);   // full[S], empty[S], acc
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * STAGES + 1);
    const uint32_t sbase = smem_u32(smem);
    const uint32_t full0 = smem_u32(bars), empty0 = full0 + 8 * STAGES, accb = full0 + 16 * STAGES;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int2 tile = a.tiles[blockIdx.x];
    const int c = blockIdx.y;
    const int i0 = tile.x, j0 = tile.y;
    const int S = a.S;
    const int nk = (a.K + BK - 1) / BK;
    // columns this tile needs: j < min(j0 + BN, i0 + BM, S), rounded up to 16
    const int n_need = min(min(j0 + BN, i0 + BM), S) - j0;
    const uint32_t n_eff = (uint32_t)((n_need + 15) & ~15);
    const bool half_b = n_eff <= (uint32_t)BM;      // only the first 128 B rows are loaded
    // a diagonal tile (i0 == j0) multiplies its rows by themselves: B is A, so
    // its stages load A only (as every tile does when S <= BM)
    const bool diag = a.small || i0 == j0;
    // and, when its stages span the full ring, its imaginary part is M - M^T
    // with M = Ai Ar^T: three MMAs per k-step instead of four, M staged through
    // shared memory for the transpose in the epilogue
    const bool mtr = diag && !a.small;
    // S < 128: the boxes hold the S (rounded up to 8) rows that exist, so a
    // channel's planes are read once; the rows of the operand tiles past them
    // only feed accumulator rows and columns that are never stored
    const uint32_t stage_tx = diag ? 2u * (uint32_t)a.box_rows * BK * 2
                              : half_b ? 4u * (uint32_t)a.box_rows * BK * 2 : STAGE_BYTES;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; s++) {
            tc::mbar_init(full0 + 8 * s, 1);
            tc::mbar_init(empty0 + 8 * s, 1);
        }
        tc::mbar_init(accb, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmap)) : "memory");
    }
    if (warp == 1) {
        tc::tmem_alloc(smem_u32(tmem_slot), a.tmem_cols);
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        // ---------------- TMA producer ----------------
        if (lane == 0) {
            const int rowA_re = (c * 2 + 0) * S + i0, rowA_im = (c * 2 + 1) * S + i0;
            const int rowB_re = (c * 2 + 0) * S + j0, rowB_im = (c * 2 + 1) * S + j0;
            // k-blocked: rows (c, s) with the plane a coordinate of its own;
            // channel-grouped: the input s a coordinate, the channel split
            // into (c % 16, c / 16), the plane as x = 32 plane halves (64 B)
            const int krowA = a.kblock == 2 ? i0 : c * S + i0, krowB = a.kblock == 2 ? j0 : c * S + j0;
            auto load = [&](uint32_t dst, int kc, int plane, int row2d, int rowk, uint32_t bar) {
                if (a.kblock == 2) tc::tma_load_5d(dst, &tmap, 32 * plane, c & 15, kc, rowk, c >> 4, bar);
                else if (a.kblock) tc::tma_load_4d(dst, &tmap, 0, plane, kc, rowk, bar);
                else tc::tma_load_2d(dst, &tmap, kc * BK, row2d, bar);
            };
            int issued = 0;
            bool ok = true;
            for (int kc = 0; kc < nk && ok; kc++) {
                const int s = kc % STAGES;
                const uint32_t ph = (kc / STAGES) & 1;
                if (!mbar_wait(empty0 + 8 * s, ph ^ 1, ERR_EMPTY_WAIT)) { ok = false; break; }
                const uint32_t st = sbase + s * stage_bytes;
                const uint32_t fb = full0 + 8 * s;
                tc::mbar_expect_tx(fb, stage_tx);
                load(st, kc, 0, rowA_re, krowA, fb);
                load(st + A_BYTES, kc, 1, rowA_im, krowA, fb);
                if (!diag) {
                    load(st + 2 * A_BYTES, kc, 0, rowB_re, krowB, fb);
                    load(st + 2 * A_BYTES + B_BYTES, kc, 1, rowB_im, krowB, fb);
                }
                if (!half_b) {
                    load(st + 2 * A_BYTES + A_BYTES, kc, 0, rowB_re + BM, krowB + BM, fb);
                    load(st + 2 * A_BYTES + B_BYTES + A_BYTES, kc, 1, rowB_im + BM, krowB + BM, fb);
                }
                issued = kc + 1;
            }
            // drain: every stage this thread filled must have landed before the CTA exits
            for (int kc = (issued > STAGES ? issued - STAGES : 0); kc < issued; kc++)
                mbar_wait(full0 + 8 * (kc % STAGES), (kc / STAGES) & 1, ERR_FULL_WAIT);
        }
    } else if (warp == 1) {
        // ---------------- MMA issuer ----------------
        if (lane == 0) {
            const uint32_t id_pos = tc::idesc_f16(BM, n_eff, false, false, false), id_neg = tc::idesc_f16(BM, n_eff, true, false, false);
            const uint32_t d_re = tmem, d_im = tmem + a.tmem_cols / 2;
            bool ok = true;
            for (int kc = 0; kc < nk; kc++) {
                const int s = kc % STAGES;
                if (!mbar_wait(full0 + 8 * s, (kc / STAGES) & 1, ERR_FULL_WAIT)) { ok = false; break; }
                tc::fence_after();
                const uint32_t st = sbase + s * stage_bytes;
#pragma unroll
                for (int kk = 0; kk < BK / 16; kk++) {
                    const uint32_t off = kk * 32;                  // 16 FP16 along K
                    const uint64_t ar = sw64_desc(st + off), ai = sw64_desc(st + A_BYTES + off);
                    const uint64_t br = diag ? ar : sw64_desc(st + 2 * A_BYTES + off);
                    const uint64_t bi = diag ? ai : sw64_desc(st + 2 * A_BYTES + B_BYTES + off);
                    const uint32_t acc = (kc | kk) ? 1u : 0u;
                    tc::mma_f16(d_re, ar, br, id_pos, acc);           // Re += Ar Br^T
                    tc::mma_f16(d_re, ai, bi, id_pos, 1u);            // Re += Ai Bi^T
                    tc::mma_f16(d_im, ai, br, id_pos, acc);           // Im += Ai Br^T  (M on a diagonal tile)
                    if (!mtr) tc::mma_f16(d_im, ar, bi, id_neg, 1u);  // Im -= Ar Bi^T
                }
                tc::commit(empty0 + 8 * s);                       // stage free once these MMAs finish
            }
            // Always commit: the barrier then completes only after every MMA
            // issued so far has finished, so TMEM is never freed under one.
            tc::commit(accb);
            if (!ok) atomicCAS(&g_tc_error, 0u, ERR_FULL_WAIT);
        }
        __syncwarp();
    } else {
        // ---------------- epilogue: TMEM -> global ----------------
        const int q = warp & 3;                                    // TMEM lane quarter
        const int r = 32 * q + lane;
        const int i = i0 + r;
        bool ok = mbar_wait(accb, 0, ERR_ACC_WAIT);
        ok = ok && (*reinterpret_cast<volatile unsigned*>(&g_tc_error) == 0u);
        __syncwarp();
        // M - M^T needs the other warps' rows: the four epilogue warps agree
        // (one vote, so all of them or none reach the barrier below)
        bool go = __all_sync(0xffffffffu, ok);
        if (mtr) go = epi_vote(go);
        if (go) {
            tc::fence_after();
            // Stage each 32-row x 16-column block through shared memory (the
            // operand ring is free once the accumulators are final) so that a
            // store instruction writes two 128-byte runs of one output row.
            float2* stg = reinterpret_cast<float2*>(smem) + (warp - 2) * 32 * 17;
            // diagonal tile: M [BM][MP] after the four warps' staging blocks
            float* msh = reinterpret_cast<float*>(smem + EPI_STG_BYTES);
            const uint32_t lane_base = tmem + ((uint32_t)(32 * q) << 16);
            const float si = (a.inv_scale && i < S) ? __ldg(a.inv_scale + (int64_t)i * a.scale_stride + c) : 1.f;
            const int ncb = (int)(n_eff / 16);
            if (mtr) {
                for (int cb = 0; cb < ncb; cb++) {
                    uint32_t mm[16];
                    tc::tmem_ld_32x32b_x16(lane_base + a.tmem_cols / 2 + cb * 16, mm);
                    tc::tmem_ld_wait();
#pragma unroll
                    for (int jj = 0; jj < 16; jj++) msh[r * MP + cb * 16 + jj] = __uint_as_float(mm[jj]);
                }
                epi_bar();
            }
            for (int cb = 0; cb < ncb; cb++) {
                uint32_t re[16], im[16];
                tc::tmem_ld_32x32b_x16(lane_base + cb * 16, re);
                if (!mtr) tc::tmem_ld_32x32b_x16(lane_base + a.tmem_cols / 2 + cb * 16, im);
                tc::tmem_ld_wait();
                if (mtr) {
#pragma unroll
                    for (int jj = 0; jj < 16; jj++) {
                        const int jl = cb * 16 + jj;                   // column within the tile
                        im[jj] = __float_as_uint(msh[r * MP + jl] - msh[jl * MP + r]);
                    }
                }
#pragma unroll
                for (int jj = 0; jj < 16; jj++) {
                    float f = si;
                    if (a.inv_scale) {
                        const int j = j0 + cb * 16 + jj;
                        f *= (j < S) ? __ldg(a.inv_scale + (int64_t)j * a.scale_stride + c) : 0.f;
                    }
                    stg[lane * 17 + jj] = make_float2(__uint_as_float(re[jj]) * f, __uint_as_float(im[jj]) * f);
                }
                __syncwarp();
#pragma unroll 4
                for (int it = 0; it < 16; it++) {
                    const int rr = 2 * it + (lane >> 4), col = lane & 15;
                    const int ii = i0 + 32 * q + rr, j = j0 + cb * 16 + col;
                    if (ii < S && j <= ii) {
                        float2 v = stg[rr * 17 + col];
                        float2* o = a.vis + (int64_t)c * a.P + (int64_t)ii * (ii + 1) / 2 + j;
                        if (a.accumulate) {
                            const float2 old = *o;
                            v.x += old.x;
                            v.y += old.y;
                        }
                        *o = v;
                    }
                }
                __syncwarp();
            }
        }
        tc::fence_before();
    }
    __syncthreads();
    if (warp == 1) {
        tc::fence_after();
        tc::tmem_dealloc(tmem, a.tmem_cols);
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
std::mutex g_tiles_mu;
std::vector<std::pair<std::pair<int, int>, int2*>> g_tiles;   // ((device, S) -> device tile list)

const int2* tile_list(int S, int* ntiles)
{
    std::vector<int2> h;
    for (int i0 = 0; i0 < S; i0 += BM)
        for (int j0 = 0; j0 < S; j0 += BN)
            if (j0 <= i0 + BM - 1) h.push_back(make_int2(i0, j0));
    *ntiles = (int)h.size();
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(g_tiles_mu);
    for (auto& e : g_tiles)
        if (e.first.first == dev && e.first.second == S) return e.second;
    int2* d = nullptr;
    if (cudaMalloc(&d, sizeof(int2) * h.size()) != cudaSuccess) return nullptr;
    cudaMemcpy(d, h.data(), sizeof(int2) * h.size(), cudaMemcpyHostToDevice);
    g_tiles.push_back({{dev, S}, d});
    return d;
}

}  // namespace

CsEncodeTiledFn cs_encode_tiled()
{
    static CsEncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<CsEncodeTiledFn>(p);
    });
    return fn;
}

int cs_xmac_tc_f16(const void* spectra, int S, int C, int K, int kp, float2* vis, const float* inv_scale,
                   int scale_stride, int accumulate, cudaStream_t st, int kblock)
{
    if (!spectra || !vis || S <= 0 || C <= 0 || K <= 0 || C > 65535 || kp < K) return CS_ERR_ARG;
    if (K % 8 != 0 || kp % 8 != 0 || (uintptr_t)spectra % 16) return CS_ERR_ARG;   // TMA: 16-byte pitch and base
    if (kblock < 0 || kblock > 2 || (kblock && (K % 32 != 0 || kp % 32 != 0)) || (kblock == 2 && C % 16 != 0))
        return CS_ERR_ARG;
    CsEncodeTiledFn enc = cs_encode_tiled();
    if (!enc) return CS_ERR_UNSUPPORTED;
    int ntiles = 0;
    const int2* tiles = tile_list(S, &ntiles);
    if (!tiles) return CS_ERR_ARG;

    CUtensorMap tm;
    cuuint64_t gdim[2] = {(cuuint64_t)K, (cuuint64_t)C * 2 * S};
    cuuint64_t gstride[1] = {(cuuint64_t)kp * 2};
    const int box_rows = S < BM ? (S + 7) / 8 * 8 : BM;
    cuuint32_t box[2] = {BK, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r;
    if (!kblock) {
        r = enc(&tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, const_cast<void*>(spectra), gdim, gstride, box, estr,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    } else if (kblock == 2) {
        // [C/16 groups][S inputs][K/32 used of kp/32 blocks][16 channels][64
        // halves (Re 32, Im 32)]: a box of (32 halves, 1 channel, 1 block,
        // box_rows inputs, 1 group) lands as the same [rows][32] tile; inputs
        // past S read as zeros
        cuuint64_t g5[5] = {64, 16, (cuuint64_t)K / 32, (cuuint64_t)S, (cuuint64_t)C / 16};
        cuuint64_t s5[4] = {128, 2048, (cuuint64_t)kp / 32 * 2048, (cuuint64_t)S * (kp / 32) * 2048};
        cuuint32_t b5[5] = {32, 1, 1, (cuuint32_t)box_rows, 1};
        cuuint32_t e5[5] = {1, 1, 1, 1, 1};
        r = enc(&tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 5, const_cast<void*>(spectra), g5, s5, b5, e5,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    } else {
        // [C*S rows][K/32 used of kp/32 blocks][2 planes][32 halves]: a box of
        // (32 halves, 1 plane, 1 block, box_rows rows) lands in shared memory as
        // the same [rows][32] tile as the channel-major map's box
        cuuint64_t g4[4] = {32, 2, (cuuint64_t)K / 32, (cuuint64_t)C * S};
        cuuint64_t s4[3] = {64, 128, (cuuint64_t)kp / 32 * 128};
        cuuint32_t b4[4] = {32, 1, 1, (cuuint32_t)box_rows};
        cuuint32_t e4[4] = {1, 1, 1, 1};
        r = enc(&tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 4, const_cast<void*>(spectra), g4, s4, b4, e4,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    }
    if (r != CUDA_SUCCESS) return CS_ERR_ARG;

    void* errp = nullptr;
    CS_CUDA_TRY(cudaGetSymbolAddress(&errp, g_tc_error));
    CS_CUDA_TRY(cudaMemsetAsync(errp, 0, sizeof(unsigned), st));

    // S <= 128: one diagonal tile per channel, B = A, 16 KB stages and only the
    // TMEM columns the tile needs, so several CTAs share an SM
    const int small = S <= BM ? 1 : 0;
    uint32_t cols = TMEM_COLS;
    if (small) {
        const uint32_t n_eff = (uint32_t)((S + 15) & ~15);
        cols = 32;
        while (cols < 2 * n_eff) cols *= 2;
    }
    TcArgs a{S, C, K, (int64_t)S * (S + 1) / 2, tiles, vis, inv_scale, scale_stride > 0 ? scale_stride : C,
             accumulate, box_rows, small, cols, kblock};
    const size_t smem = (size_t)STAGES * (small ? 2 * A_BYTES : STAGE_BYTES) + 1024 + 256;
    CS_CUDA_TRY(cs_smem_at_least(reinterpret_cast<const void*>(k_xmac_tc), (int)smem));
    dim3 grid(ntiles, C);
    k_xmac_tc<<<grid, TC_THREADS, smem, st>>>(tm, a), cs_count_launches(1);
    return (int)cudaGetLastError();
}

// Error code of the last tensor-core launch on this device (0 = ok); the
// caller must have synchronised the launching stream.
int cs_xmac_tc_status(unsigned* code)
{
    return (int)cudaMemcpyFromSymbol(code, g_tc_error, sizeof(unsigned));
}
