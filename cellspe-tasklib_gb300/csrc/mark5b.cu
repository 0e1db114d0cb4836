// Framed Mark5B input: frame search, fill-pattern blanking, deframing.
//
// A Mark5B recording is a sequence of 10016-byte frames: a 16-byte header
// starting with the sync word 0xABADDEED, then 10000 bytes of payload
// (mark5_format_mark5b.c:2817-2819).  Missing data is recorded as the fill
// pattern 0x11223344; mark5access blanks it per payload with blanker_mark5
// (blanker_mark5.c): if the first and last 64-bit words are data the whole
// payload is valid, if both are fill it is blanked, otherwise a binary search
// finds the boundary; blanked samples decode as 0.0.  The kernels below apply
// exactly these rules (the search steps included, so partially filled words
// resolve the same way) and the first-frame rule of findfirstframe
// (mark5_format_mark5b.c:98-131: the sync word twice, 10016 bytes apart,
// within the first MiB).  Frame f is present when its 10016 bytes lie inside
// the buffer; the frame offset lives on the device, so no launch here waits
// for the host.
//
// Sample time t of an nch-channel 2-bit stream sits in frame t / spf at
// payload byte (t % spf) * bps, bps = nch / 4 bytes per sample time,
// spf = 10000 / bps; channel c is bits 2(c%4)..2(c%4)+1 of byte c/4.
#include "common.cuh"
#include "kernels.h"

namespace {

constexpr int FRAME = 10016, PAYLOAD = 10000, SCAN_LIMIT = 1 << 20;
constexpr unsigned long long FILL64 = 0x1122334411223344ULL;
constexpr unsigned FILL32 = 0x11223344u;

CS_DEV uint64_t ld64(const uint8_t* p, int64_t w)
{
    uint64_t v = 0;
#pragma unroll
    for (int b = 7; b >= 0; b--) v = (v << 8) | p[8 * w + b];
    return v;
}
CS_DEV uint32_t ld32(const uint8_t* p, int64_t w)
{
    return (uint32_t)p[4 * w] | ((uint32_t)p[4 * w + 1] << 8) | ((uint32_t)p[4 * w + 2] << 16) |
           ((uint32_t)p[4 * w + 3] << 24);
}

// true when frame f of the stream starting at off lies inside the buffer
CS_DEV bool frame_present(int64_t off, int64_t f, int64_t bytes)
{
    return off < SCAN_LIMIT && off + (f + 1) * FRAME <= bytes;
}

__global__ void k_first_frame(const uint8_t* __restrict__ d, int64_t nscan, int* __restrict__ result)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nscan) return;
    if (d[i] == 0xED && d[i + 1] == 0xDE && d[i + 2] == 0xAD && d[i + 3] == 0xAB && d[i + FRAME] == 0xED &&
        d[i + FRAME + 1] == 0xDE && d[i + FRAME + 2] == 0xAD && d[i + FRAME + 3] == 0xAB)
        atomicMin(result, (int)i);
}

// blanker_mark5.c binary searches over the n 64-bit words of one payload
CS_DEV int first_invalid(const uint8_t* p, int n)
{
    int i = n / 2, r = n - 1;
    for (int s = n / 4; s > 0; s >>= 1) {
        if (ld64(p, i) == FILL64) { r = i; i -= s; }
        else i += s;
    }
    r = 8 * r;
    if (ld32(p, r / 4 - 1) == FILL32) r -= 4;
    return r;
}

CS_DEV int first_valid(const uint8_t* p, int n)
{
    int i = n / 2, r = n - 1;
    for (int s = n / 4; s > 0; s >>= 1) {
        if (ld64(p, i) != FILL64) { r = i; i -= s; }
        else i += s;
    }
    r = 8 * r;
    if (ld32(p, r / 4 - 2) == FILL32) r += 4;
    return r;
}

// one thread per frame: valid payload byte range [x, y); absent frames blank
__global__ void k_valid_ranges(const uint8_t* __restrict__ framed, int64_t bytes, const int* __restrict__ offset,
                               int64_t nframes, int2* __restrict__ ranges)
{
    int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nframes) return;
    const int64_t off = *offset;
    int2 r = make_int2(1 << 30, 0);
    if (frame_present(off, f, bytes)) {
        const uint8_t* p = framed + off + f * FRAME + 16;
        const int nword = PAYLOAD / 8;
        const bool s_ok = ld64(p, 0) != FILL64, e_ok = ld64(p, nword - 1) != FILL64;
        if (s_ok && e_ok) r = make_int2(0, 1 << 30);
        else if (s_ok) r = make_int2(0, first_invalid(p, nword));
        else if (e_ok) r = make_int2(first_valid(p, nword), 1 << 30);
    }
    ranges[f] = r;
}

// mark5_stream_decode: thread per sample time, nch float planes, 0.0 in
// blanked zones, nothing written past the last present frame; counts the
// unblanked samples
__global__ void k_decode_framed(const uint8_t* __restrict__ framed, int64_t bytes, const int* __restrict__ offset,
                                const int2* __restrict__ ranges, int nch, int64_t nsamp, float* __restrict__ out,
                                float l0, float l1, float l2, float l3, unsigned long long* __restrict__ good)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int bps = nch / 4, spf = PAYLOAD / bps;
    const int64_t off = *offset;
    const int64_t f = t / spf;
    const bool live = t < nsamp && frame_present(off, f, bytes);
    bool valid = false;
    if (live) {
        const int i = (int)(t - f * spf) * bps;
        const int2 r = ranges[f];
        valid = i >= r.x && i < r.y;
        const uint8_t* p = framed + off + f * FRAME + 16 + i;
        const float lut[4] = {l0, l1, l2, l3};
        for (int b = 0; b < bps; b++) {
            const unsigned byte = p[b];
#pragma unroll
            for (int q = 0; q < 4; q++)
                out[(int64_t)(4 * b + q) * nsamp + t] = valid ? lut[(byte >> (2 * q)) & 3u] : 0.0f;
        }
    }
    const unsigned n = __popc(__ballot_sync(0xffffffffu, valid));
    if ((threadIdx.x & 31) == 0 && n) atomicAdd(good, (unsigned long long)n);
}

// FileSource::read for framed data: payload words of every frame back to
// back (thread per 32-bit output word; absent frames give zeros)
__global__ void k_deframe(const uint8_t* __restrict__ framed, int64_t bytes, const int* __restrict__ offset,
                          int64_t nframes, uint32_t* __restrict__ payload)
{
    const int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    constexpr int WPF = PAYLOAD / 4;
    if (w >= nframes * WPF) return;
    const int64_t off = *offset;
    const int64_t f = w / WPF;
    uint32_t v = 0;
    if (frame_present(off, f, bytes)) v = ld32(framed + off + f * FRAME + 16, w - f * WPF);
    payload[w] = v;
}

// validity bit per sample time: bit t%32 of word t/32 set = sample t is data
__global__ void k_valid_mask(const int2* __restrict__ ranges, int64_t nframes, int bps, int64_t nwords,
                             uint32_t* __restrict__ mask)
{
    const int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= nwords) return;
    const int spf = PAYLOAD / bps;
    uint32_t bits = 0;
    for (int q = 0; q < 32; q++) {
        const int64_t t = 32 * w + q, f = t / spf;
        if (f >= nframes) break;
        const int i = (int)(t - f * spf) * bps;
        const int2 r = ranges[f];
        bits |= (uint32_t)(i >= r.x && i < r.y) << q;
    }
    mask[w] = bits;
}

// Deframe + corner turn + validity mask in one pass: thread per group of 16
// sample times writes one 32-bit word (16 2-bit codes) of each channel plane
// and 16 validity bits; neighbouring lanes pair their bits into mask words.
// Groups past the last present frame give zero codes and clear bits.
template <int NCH>
__global__ void k_deframe_planes(const uint8_t* __restrict__ framed, int64_t bytes, const int* __restrict__ offset,
                                 const int2* __restrict__ ranges, int64_t nframes, int64_t ngroups,
                                 uint32_t* __restrict__ planes, uint32_t* __restrict__ mask)
{
    constexpr int BPS = NCH / 4, SPF = PAYLOAD / BPS;
    const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t off = *offset;
    uint32_t words[NCH];
#pragma unroll
    for (int c = 0; c < NCH; c++) words[c] = 0;
    uint32_t vbits = 0;
    if (g < ngroups) {
        for (int q = 0; q < 16; q++) {
            const int64_t t = 16 * g + q, f = t / SPF;
            if (f >= nframes || !frame_present(off, f, bytes)) break;
            const int i = (int)(t - f * SPF) * BPS;
            const int2 r = ranges[f];
            vbits |= (uint32_t)(i >= r.x && i < r.y) << q;
            const uint8_t* p = framed + off + f * FRAME + 16 + i;
#pragma unroll
            for (int b = 0; b < BPS; b++) {
                const uint32_t byte = p[b];
#pragma unroll
                for (int k = 0; k < 4; k++) words[4 * b + k] |= ((byte >> (2 * k)) & 3u) << (2 * q);
            }
        }
    }
    const uint32_t hi = __shfl_down_sync(0xffffffffu, vbits, 1);
    if (g < ngroups) {
        const int64_t plane_words = ngroups;
#pragma unroll
        for (int c = 0; c < NCH; c++) planes[c * plane_words + g] = words[c];
        if ((g & 1) == 0) mask[g >> 1] = vbits | ((g + 1 < ngroups ? hi : 0u) << 16);
    }
}

inline unsigned blocks_for(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

int cs_m5b_locate(const uint8_t* framed, int64_t bytes, int* d_offset, int2* ranges, int64_t nframes,
                  cudaStream_t st)
{
    if (!framed || !d_offset || !ranges || bytes < 2 * FRAME || nframes <= 0) return CS_ERR_ARG;
    // sync word at i and i + 10016 inside the buffer and the first MiB
    const int64_t nscan = (bytes < SCAN_LIMIT ? bytes : (int64_t)SCAN_LIMIT) - (FRAME + 4);
    if (nscan <= 0) return CS_ERR_ARG;
    CS_CUDA_TRY(cudaMemsetAsync(d_offset, 0x7f, sizeof(int), st));
    k_first_frame<<<blocks_for(nscan, 256), 256, 0, st>>>(framed, nscan, d_offset), cs_count_launches(1);
    k_valid_ranges<<<blocks_for(nframes, 128), 128, 0, st>>>(framed, bytes, d_offset, nframes, ranges),
        cs_count_launches(1);
    return (int)cudaGetLastError();
}

int cs_m5b_decode(const uint8_t* framed, int64_t bytes, const int* d_offset, const int2* ranges, int nch,
                  int64_t nsamp, const float lut[4], float* out, unsigned long long* d_good, cudaStream_t st)
{
    if (!(nch == 4 || nch == 8 || nch == 16) || nsamp <= 0 || !out || !d_good) return CS_ERR_ARG;
    CS_CUDA_TRY(cudaMemsetAsync(d_good, 0, sizeof(unsigned long long), st));
    k_decode_framed<<<blocks_for(nsamp, 256), 256, 0, st>>>(framed, bytes, d_offset, ranges, nch, nsamp, out, lut[0],
                                                           lut[1], lut[2], lut[3], d_good),
        cs_count_launches(1);
    return (int)cudaGetLastError();
}

int cs_m5b_deframe(const uint8_t* framed, int64_t bytes, const int* d_offset, const int2* ranges, int64_t nframes,
                   int nch, uint8_t* payload, uint32_t* mask, cudaStream_t st)
{
    if (!(nch == 4 || nch == 8 || nch == 16) || nframes <= 0 || !payload) return CS_ERR_ARG;
    if ((uintptr_t)payload % 4 || ((uintptr_t)mask % 4)) return CS_ERR_ARG;
    const int bps = nch / 4;
    const int64_t nwords = nframes * (PAYLOAD / 4);
    k_deframe<<<blocks_for(nwords, 256), 256, 0, st>>>(framed, bytes, d_offset, nframes, (uint32_t*)payload),
        cs_count_launches(1);
    if (mask) {
        const int64_t nsamp = nframes * (PAYLOAD / bps), mwords = (nsamp + 31) / 32;
        k_valid_mask<<<blocks_for(mwords, 256), 256, 0, st>>>(ranges, nframes, bps, mwords, mask),
            cs_count_launches(1);
    }
    return (int)cudaGetLastError();
}

int cs_m5b_planes(const uint8_t* framed, int64_t bytes, const int* d_offset, const int2* ranges, int64_t nframes,
                  int nch, int64_t ngroups, uint32_t* planes, uint32_t* mask, cudaStream_t st)
{
    if (ngroups <= 0 || !planes || !mask) return CS_ERR_ARG;
    const unsigned nb = blocks_for(ngroups, 256);
    switch (nch) {
        case 4: k_deframe_planes<4><<<nb, 256, 0, st>>>(framed, bytes, d_offset, ranges, nframes, ngroups, planes, mask); break;
        case 8: k_deframe_planes<8><<<nb, 256, 0, st>>>(framed, bytes, d_offset, ranges, nframes, ngroups, planes, mask); break;
        case 16: k_deframe_planes<16><<<nb, 256, 0, st>>>(framed, bytes, d_offset, ranges, nframes, ngroups, planes, mask); break;
        default: return CS_ERR_ARG;
    }
    cs_count_launches(1);
    return (int)cudaGetLastError();
}
