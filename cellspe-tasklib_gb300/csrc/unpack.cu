// K-a: 2-bit unpack and corner turn.
//
// Decode semantics (bit-exact with the reference):
//   field (t, c) of an nchan-channel stream sits at bit 2*(t*nchan + c) of the
//   little-endian byte stream; code = bit0 + 2*bit1; value = lut[code].
//   Mark5B (mark5_format_mark5b.c:59-95, :1852-1915): lut {-H, +1, -1, +H},
//   H = 3.3359f, nchan = 16/8/4.  TwoBitUnpacker (DataUnpackers.cpp:174-227):
//   lut {1, -1, H, -H}.  Single-channel MSB-first order
//   (DataUnpackers.cpp:244-288, intended behaviour; the reference masks
//   0xC0 for every sample, an out-of-range read for samples 1..3).
//
// A warp takes 512 raw bytes (32 16-byte vectors, one coalesced load each),
// parks them in shared memory and writes every channel's float4 runs so that
// one store instruction covers 512 contiguous output bytes: the bytes holding
// sample times 4q..4q+3 of all channels (nchan bytes) feed run q, lane q mod 32.
// Levels come from register selects on the code's two bits, not from an
// indexed table load.
#include "common.cuh"
#include "kernels.h"

struct Lut4 { float v[4]; };

template <int NCH, bool MSB>
__global__ void __launch_bounds__(256) k_unpack2bit(const uint4* __restrict__ raw, int64_t nblk,
                                                    float* __restrict__ out, int64_t nsamp, Lut4 lut)
{
    constexpr int TPV = 64 / NCH;   // sample times per 16-byte vector
    constexpr int NQ = 16 / NCH;    // float4 runs per channel and lane
    __shared__ uint4 stage[8][32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int64_t blk = (int64_t)blockIdx.x * 8 + wid;   // warp block: 512 bytes, 32 * TPV sample times
    if (blk >= nblk) return;                              // whole warps leave together
    const float L0 = lut.v[0], L1 = lut.v[1], L2 = lut.v[2], L3 = lut.v[3];
    const uint4 v = __ldg(raw + blk * 32 + lane);
    if constexpr (NCH < 16) {
        stage[wid][lane] = v;
        __syncwarp();
    }
    const uint8_t* sb = reinterpret_cast<const uint8_t*>(stage[wid]);
    float* o = out + blk * 32 * TPV;
#pragma unroll
    for (int j = 0; j < NQ; j++) {
        const int q = j * 32 + lane;                      // run: sample times 4q..4q+3 of the block
        uint32_t w[4] = {0u, 0u, 0u, 0u};
        if constexpr (NCH == 16) { w[0] = v.x; w[1] = v.y; w[2] = v.z; w[3] = v.w; }
        else if constexpr (NCH == 8) { uint2 x = reinterpret_cast<const uint2*>(sb)[q]; w[0] = x.x; w[1] = x.y; }
        else if constexpr (NCH == 4) w[0] = reinterpret_cast<const uint32_t*>(sb)[q];
        else if constexpr (NCH == 2) w[0] = reinterpret_cast<const uint16_t*>(sb)[q];
        else w[0] = sb[q];
#pragma unroll
        for (int c = 0; c < NCH; c++) {
            float r[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const int f = u * NCH + c;                // field index inside the nchan-byte chunk
                const uint32_t code = code2(w[f >> 4], f & 15, MSB);
                const float lo = (code & 1u) ? L1 : L0, hi = (code & 1u) ? L3 : L2;
                r[u] = (code & 2u) ? hi : lo;
            }
            *reinterpret_cast<float4*>(o + (int64_t)c * nsamp + 4 * q) = make_float4(r[0], r[1], r[2], r[3]);
        }
    }
}

// Tail (and unaligned) path: one thread per (sample time, channel).
__global__ void k_unpack2bit_scalar(const uint8_t* __restrict__ raw, int64_t t_begin, int64_t nsamp,
                                    int nch, int msb, float* __restrict__ out, Lut4 lut)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t n = (nsamp - t_begin) * nch;
    if (i >= n) return;
    int64_t t = t_begin + i / nch;
    int c = (int)(i % nch);
    int64_t f = t * nch + c;
    uint8_t b = raw[f >> 2];
    int pos = (int)(f & 3);
    int sh = msb ? (6 - 2 * pos) : (2 * pos);
    out[(int64_t)c * nsamp + t] = lut.v[(b >> sh) & 3];
}

template <int NCH, bool MSB>
static void launch_vec(const void* raw, int64_t nblk, float* out, int64_t nsamp, Lut4 lut, cudaStream_t st)
{
    if (nblk <= 0) return;
    int64_t blocks = (nblk + 7) / 8;
    k_unpack2bit<NCH, MSB><<<(unsigned)blocks, 256, 0, st>>>((const uint4*)raw, nblk, out, nsamp, lut), cs_count_launches(1);
}

int cs_unpack2bit(const void* raw, int64_t nsamp, int nchan, int msb_first, const float lut4[4],
                  float* out, cudaStream_t st)
{
    if (nsamp < 0 || !raw || !out) return CS_ERR_ARG;
    if (!(nchan == 1 || nchan == 2 || nchan == 4 || nchan == 8 || nchan == 16)) return CS_ERR_ARG;
    if (msb_first && nchan != 1) return CS_ERR_ARG;
    Lut4 lut = {{lut4[0], lut4[1], lut4[2], lut4[3]}};
    const int tpv = 64 / nchan;
    bool aligned = ((uintptr_t)raw % 16 == 0) && ((uintptr_t)out % 16 == 0) &&
                   (nsamp % 4 == 0 || tpv < 4);
    int64_t nblk = aligned ? nsamp / tpv / 32 : 0;   // whole 512-byte warp blocks
    if (nblk > 0) {
        if (msb_first) launch_vec<1, true>(raw, nblk, out, nsamp, lut, st);
        else switch (nchan) {
            case 1: launch_vec<1, false>(raw, nblk, out, nsamp, lut, st); break;
            case 2: launch_vec<2, false>(raw, nblk, out, nsamp, lut, st); break;
            case 4: launch_vec<4, false>(raw, nblk, out, nsamp, lut, st); break;
            case 8: launch_vec<8, false>(raw, nblk, out, nsamp, lut, st); break;
            default: launch_vec<16, false>(raw, nblk, out, nsamp, lut, st); break;
        }
    }
    int64_t t_begin = nblk * 32 * tpv;
    int64_t rem = (nsamp - t_begin) * nchan;
    if (rem > 0) {
        int64_t blocks = (rem + 255) / 256;
        k_unpack2bit_scalar<<<(unsigned)blocks, 256, 0, st>>>((const uint8_t*)raw, t_begin, nsamp, nchan,
                                                              msb_first, out, lut), cs_count_launches(1);
    }
    return (int)cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Corner turn: nchan-channel interleaved 2-bit words -> one packed 2-bit
// plane per channel (4 samples per byte, LSB first).  This is the bit-plane
// separation of cornerturn (cellspe-tasklib-dsp.cpp:831-859) at 2 bits per
// field, done once so that per-subband FFT kernels read 0.25 B per sample
// instead of the whole multi-channel word.  Each thread turns 16 sample
// times: it reads 16*nchan/4 bytes and writes one 32-bit word per channel.
// ---------------------------------------------------------------------------
template <int NCH>
__global__ void __launch_bounds__(256) k_cornerturn(const uint32_t* __restrict__ in, int64_t ngroups,
                                                    uint32_t* __restrict__ planes, int64_t plane_words)
{
    constexpr int WPG = NCH;          // 32-bit input words per 16 sample times (NCH*16*2/32)
    int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ngroups) return;
    uint32_t w[WPG];
    const uint4* src = reinterpret_cast<const uint4*>(in + g * WPG);
#pragma unroll
    for (int i = 0; i < WPG / 4; i++) {
        uint4 q = __ldg(src + i);
        w[4 * i] = q.x; w[4 * i + 1] = q.y; w[4 * i + 2] = q.z; w[4 * i + 3] = q.w;
    }
    if constexpr (NCH == 16) {
        // Word t holds channel c at bits 2c; plane word c wants time t at bits 2t: a
        // 16 x 16 transpose of 2-bit fields, done as four stages of masked swaps of
        // 8-, 4-, 2- and 1-field blocks between words r and r + j.
#pragma unroll
        for (int s = 0; s < 4; s++) {
            const int j = 8 >> s;
            const uint32_t m = s == 0 ? 0x0000FFFFu : s == 1 ? 0x00FF00FFu : s == 2 ? 0x0F0F0F0Fu : 0x33333333u;
#pragma unroll
            for (int r = 0; r < 16; r++) {
                if (r & j) continue;
                const uint32_t t = ((w[r] >> (2 * j)) ^ w[r + j]) & m;
                w[r + j] ^= t;
                w[r] ^= t << (2 * j);
            }
        }
#pragma unroll
        for (int c = 0; c < 16; c++) planes[(int64_t)c * plane_words + g] = w[c];
    } else {
#pragma unroll
        for (int c = 0; c < NCH; c++) {
            uint32_t o = 0;
#pragma unroll
            for (int t = 0; t < 16; t++) {
                int f = t * NCH + c;
                o |= ((w[f >> 4] >> (2 * (f & 15))) & 3u) << (2 * t);
            }
            planes[(int64_t)c * plane_words + g] = o;
        }
    }
}

int cs_cornerturn2bit(const void* raw, int64_t nsamp, int nchan, void* planes, cudaStream_t st)
{
    if (!(nchan == 4 || nchan == 8 || nchan == 16)) return CS_ERR_ARG;
    if (nsamp % 16 != 0 || (uintptr_t)raw % 16 || (uintptr_t)planes % 16) return CS_ERR_ARG;
    int64_t groups = nsamp / 16;
    int64_t plane_words = nsamp / 16;
    int64_t blocks = (groups + 255) / 256;
    if (blocks == 0) return 0;
    switch (nchan) {
        case 4: k_cornerturn<4><<<(unsigned)blocks, 256, 0, st>>>((const uint32_t*)raw, groups, (uint32_t*)planes, plane_words), cs_count_launches(1); break;
        case 8: k_cornerturn<8><<<(unsigned)blocks, 256, 0, st>>>((const uint32_t*)raw, groups, (uint32_t*)planes, plane_words), cs_count_launches(1); break;
        default: k_cornerturn<16><<<(unsigned)blocks, 256, 0, st>>>((const uint32_t*)raw, groups, (uint32_t*)planes, plane_words), cs_count_launches(1); break;
    }
    return (int)cudaGetLastError();
}
