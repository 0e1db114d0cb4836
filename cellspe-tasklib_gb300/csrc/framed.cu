// Framed 2-bit input on the device: Mark5B and VDIF.
//
// Mark5B (mark5access mark5_format_mark5b.c): 10016-byte frames, a 16-byte
// header starting with the sync word 0xABADDEED, then 10000 bytes of payload
// (:2817-2819).  Missing data is recorded as the fill pattern 0x11223344;
// mark5access blanks it per payload with blanker_mark5 (blanker_mark5.c): if
// the first and last 64-bit words are data the whole payload is valid, if both
// are fill it is blanked, otherwise a binary search finds the boundary;
// blanked samples decode as 0.0.  The kernels apply exactly these rules (the
// search steps included, so partially filled words resolve the same way) and
// the first-frame rule of findfirstframe (:98-131: the sync word twice, 10016
// bytes apart, within the first MiB).  The frame offset lives on the device,
// so no launch here waits for the host.
//
// VDIF (format_vdif.c): frames from byte 0, the frame length in the first
// header.  A frame is used whole or blanked whole: frames after the first are
// blanked when their header time is not the one predicted from the first
// frame (checked on frame numbers that are multiples of the frame-time
// granularity, mark5_format_vdif_validate :2299-2337) or the invalid bit is
// set; every frame is blanked when its first or last 64-bit payload word is
// fill (blanker_vdif, blanker_mark5.c:282-316).
//
// Both formats: sample time t of an nch-channel 2-bit stream sits in frame
// t / spf, spf = payload_bytes * 4 / nch; channel c of it is the 2-bit field
// at bit 2 * ((t % spf) * nch + c) of the payload (little-endian bit order);
// the byte holding the field's first bit decides blanking.  Frame f is present
// when its bytes lie inside the buffer.
#include "common.cuh"
#include "kernels.h"

namespace {

constexpr int M5B_FRAME = 10016, M5B_PAYLOAD = 10000, SCAN_LIMIT = 1 << 20;
constexpr unsigned long long FILL64 = 0x1122334411223344ULL;
constexpr unsigned FILL32 = 0x11223344u;
constexpr int BLANK_ALL = 1 << 30;

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

CS_DEV int64_t stream_offset(const int* offset) { return offset ? (int64_t)*offset : 0; }

// true when frame f of the stream starting at off lies inside the buffer
CS_DEV bool frame_present(const CsFraming& fm, int64_t off, int64_t f, int64_t bytes)
{
    return off < SCAN_LIMIT && off + (f + 1) * fm.frame_bytes <= bytes;
}

CS_DEV const uint8_t* payload_of(const uint8_t* framed, const CsFraming& fm, int64_t off, int64_t f)
{
    return framed + off + f * fm.frame_bytes + (f == 0 ? fm.frame0_payload_offset : fm.payload_offset);
}

__global__ void k_first_frame(const uint8_t* __restrict__ d, int64_t nscan, int* __restrict__ result)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nscan) return;
    if (d[i] == 0xED && d[i + 1] == 0xDE && d[i + 2] == 0xAD && d[i + 3] == 0xAB && d[i + M5B_FRAME] == 0xED &&
        d[i + M5B_FRAME + 1] == 0xDE && d[i + M5B_FRAME + 2] == 0xAD && d[i + M5B_FRAME + 3] == 0xAB)
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

// Mark5B, one thread per frame: valid payload byte range [x, y); absent
// frames blank
__global__ void k_m5b_ranges(const uint8_t* __restrict__ framed, int64_t bytes, const int* __restrict__ offset,
                             int64_t nframes, int2* __restrict__ ranges)
{
    int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nframes) return;
    const int64_t off = *offset;
    const CsFraming fm{M5B_FRAME, M5B_PAYLOAD, 16, 16, 0};
    int2 r = make_int2(BLANK_ALL, 0);
    if (frame_present(fm, off, f, bytes)) {
        const uint8_t* p = payload_of(framed, fm, off, f);
        const int nword = M5B_PAYLOAD / 8;
        const bool s_ok = ld64(p, 0) != FILL64, e_ok = ld64(p, nword - 1) != FILL64;
        if (s_ok && e_ok) r = make_int2(0, BLANK_ALL);
        else if (s_ok) r = make_int2(0, first_invalid(p, nword));
        else if (e_ok) r = make_int2(first_valid(p, nword), BLANK_ALL);
    }
    ranges[f] = r;
}

// VDIF header time of one frame (mark5_stream_frame_time_vdif, no leap
// seconds): MJD, seconds of day, nanoseconds of frame number * frame_ns
CS_DEV void vdif_time(const uint8_t* h, const CsVdifClock& c, int& mjd, int& sec, double& ns)
{
    const uint32_t w0 = ld32(h, 0), w1 = ld32(h, 1);
    int seconds = (int)(w0 & 0x3FFFFFFFu);
    const int days = seconds / 86400;
    seconds -= days * 86400;
    mjd = days + c.epoch_mjd[(w1 >> 24) & 0x3F];
    sec = seconds;
    ns = (double)(w1 & 0x00FFFFFFu) * c.frame_ns;
}

// VDIF, one thread per frame: (0, all) when the frame is used, (all, 0) when
// it is blanked; blanked frames (absent ones included) are counted
__global__ void k_vdif_ranges(const uint8_t* __restrict__ framed, int64_t bytes, const __grid_constant__ CsVdifClock c,
                              int64_t nframes, int2* __restrict__ ranges, unsigned long long* __restrict__ blanked)
{
    const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool ok = false;
    if (f < nframes && frame_present(c.fmt, 0, f, bytes)) {
        const uint8_t* h = framed + f * c.fmt.frame_bytes;
        ok = true;
        if (f > 0) {
            if (c.mjd0 != 0 && f % c.granularity == 0) {
                int mjd_d, sec_d;
                double ns_d;
                vdif_time(h, c, mjd_d, sec_d, ns_d);
                long long ns_t = (long long)f * c.step_ns + (long long)c.ns0;
                int sec_t = (int)(ns_t / 1000000000LL);
                ns_t -= (long long)sec_t * 1000000000LL;
                sec_t += c.sec0;
                int mjd_t = sec_t / 86400;
                sec_t -= mjd_t * 86400;
                mjd_t += c.mjd0;
                if (mjd_t != mjd_d || sec_t != sec_d || fabs((double)ns_t - ns_d) > 0.000001) ok = false;
            }
            if ((ld32(h, 0) >> 31) & 1u) ok = false;
        }
        if (ok) {
            const uint8_t* p = payload_of(framed, c.fmt, 0, f);
            const int nword = c.fmt.payload_bytes / 8;
            if (ld64(p, 0) == FILL64 || ld64(p, nword - 1) == FILL64) ok = false;
        }
    }
    if (f < nframes) ranges[f] = ok ? make_int2(0, BLANK_ALL) : make_int2(BLANK_ALL, 0);
    const unsigned n = __popc(__ballot_sync(0xffffffffu, f < nframes && !ok));
    if ((threadIdx.x & 31) == 0 && n) atomicAdd(blanked, (unsigned long long)n);
}

// 2-bit code of channel c at sample s of a payload
CS_DEV unsigned code_at(const uint8_t* p, int64_t s, int nch, int c)
{
    const int64_t bit = 2 * (s * nch + c);
    return (p[bit >> 3] >> (bit & 7)) & 3u;
}

// mark5_stream_decode: thread per sample time, nch float planes, 0.0 in
// blanked zones, nothing written past the last present frame; counts the
// unblanked samples
__global__ void k_decode_framed(const uint8_t* __restrict__ framed, int64_t bytes, const CsFraming fm,
                                const int* __restrict__ offset, const int2* __restrict__ ranges, int64_t nsamp,
                                float l0, float l1, float l2, float l3, float* __restrict__ out,
                                unsigned long long* __restrict__ good)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t spf = (int64_t)fm.payload_bytes * 4 / fm.nch;
    const int64_t off = stream_offset(offset);
    const int64_t f = t / spf;
    const bool live = t < nsamp && frame_present(fm, off, f, bytes);
    bool valid = false;
    if (live) {
        const int64_t s = t - f * spf;
        const int i = (int)((2 * s * fm.nch) >> 3);
        const int2 r = ranges[f];
        valid = i >= r.x && i < r.y;
        const uint8_t* p = payload_of(framed, fm, off, f);
        const float lut[4] = {l0, l1, l2, l3};
        for (int c = 0; c < fm.nch; c++) out[(int64_t)c * nsamp + t] = valid ? lut[code_at(p, s, fm.nch, c)] : 0.0f;
    }
    const unsigned n = __popc(__ballot_sync(0xffffffffu, valid));
    if ((threadIdx.x & 31) == 0 && n) atomicAdd(good, (unsigned long long)n);
}

// payload words of every frame back to back (thread per 32-bit output word;
// absent frames give zeros)
__global__ void k_deframe(const uint8_t* __restrict__ framed, int64_t bytes, const CsFraming fm,
                          const int* __restrict__ offset, int64_t nframes, uint32_t* __restrict__ payload)
{
    const int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int wpf = fm.payload_bytes / 4;
    if (w >= nframes * wpf) return;
    const int64_t off = stream_offset(offset);
    const int64_t f = w / wpf;
    uint32_t v = 0;
    if (frame_present(fm, off, f, bytes)) v = ld32(payload_of(framed, fm, off, f), w - f * wpf);
    payload[w] = v;
}

// validity bit per sample time: bit t%32 of word t/32 set = sample t is data
__global__ void k_valid_mask(const int2* __restrict__ ranges, const CsFraming fm, int64_t nframes, int64_t nwords,
                             uint32_t* __restrict__ mask)
{
    const int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= nwords) return;
    const int64_t spf = (int64_t)fm.payload_bytes * 4 / fm.nch;
    uint32_t bits = 0;
    for (int q = 0; q < 32; q++) {
        const int64_t t = 32 * w + q, f = t / spf;
        if (f >= nframes) break;
        const int i = (int)((2 * (t - f * spf) * fm.nch) >> 3);
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
__global__ void k_deframe_planes(const uint8_t* __restrict__ framed, int64_t bytes, const CsFraming fm,
                                 const int* __restrict__ offset, const int2* __restrict__ ranges, int64_t nframes,
                                 int64_t ngroups, uint32_t* __restrict__ planes, uint32_t* __restrict__ mask)
{
    const int64_t spf = (int64_t)fm.payload_bytes * 4 / NCH;
    const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t off = stream_offset(offset);
    uint32_t words[NCH];
#pragma unroll
    for (int c = 0; c < NCH; c++) words[c] = 0;
    uint32_t vbits = 0;
    if (g < ngroups) {
        for (int q = 0; q < 16; q++) {
            const int64_t t = 16 * g + q, f = t / spf;
            if (f >= nframes || !frame_present(fm, off, f, bytes)) break;
            const int64_t s = t - f * spf;
            const int i = (int)((2 * s * NCH) >> 3);
            const int2 r = ranges[f];
            vbits |= (uint32_t)(i >= r.x && i < r.y) << q;
            const uint8_t* p = payload_of(framed, fm, off, f);
            if constexpr (NCH >= 4) {
                const uint8_t* b = p + i;
#pragma unroll
                for (int k = 0; k < NCH / 4; k++) {
                    const uint32_t byte = b[k];
#pragma unroll
                    for (int j = 0; j < 4; j++) words[4 * k + j] |= ((byte >> (2 * j)) & 3u) << (2 * q);
                }
            } else {
#pragma unroll
                for (int c = 0; c < NCH; c++) words[c] |= code_at(p, s, NCH, c) << (2 * q);
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

// Geometry checks; the payload of frame 0 may start past the frame header
// (a legacy VDIF stream opened with 32-byte headers) but must end inside the
// buffer, and every other payload inside its frame.
bool framing_ok(const CsFraming& fm, int64_t bytes)
{
    const bool nch_ok = fm.nch == 1 || fm.nch == 2 || fm.nch == 4 || fm.nch == 8 || fm.nch == 16;
    return nch_ok && fm.payload_bytes >= 8 && fm.payload_bytes % 8 == 0 && fm.frame_bytes > 0 &&
           (int64_t)fm.payload_bytes * 4 % fm.nch == 0 && fm.payload_offset >= 0 &&
           fm.payload_offset + (int64_t)fm.payload_bytes <= fm.frame_bytes && fm.frame0_payload_offset >= 0 &&
           fm.frame0_payload_offset + (int64_t)fm.payload_bytes <= bytes;
}

}  // namespace

int cs_m5b_locate(const uint8_t* framed, int64_t bytes, int* d_offset, int2* ranges, int64_t nframes,
                  cudaStream_t st)
{
    if (!framed || !d_offset || !ranges || bytes < 2 * M5B_FRAME || nframes <= 0) return CS_ERR_ARG;
    // sync word at i and i + 10016 inside the buffer and the first MiB
    const int64_t nscan = (bytes < SCAN_LIMIT ? bytes : (int64_t)SCAN_LIMIT) - (M5B_FRAME + 4);
    if (nscan <= 0) return CS_ERR_ARG;
    CS_CUDA_TRY(cudaMemsetAsync(d_offset, 0x7f, sizeof(int), st));
    k_first_frame<<<blocks_for(nscan, 256), 256, 0, st>>>(framed, nscan, d_offset), cs_count_launches(1);
    k_m5b_ranges<<<blocks_for(nframes, 128), 128, 0, st>>>(framed, bytes, d_offset, nframes, ranges),
        cs_count_launches(1);
    return (int)cudaGetLastError();
}

int cs_vdif_locate(const uint8_t* framed, int64_t bytes, const CsVdifClock& clk, int2* ranges, int64_t nframes,
                   unsigned long long* d_blanked, cudaStream_t st)
{
    if (!framed || !ranges || !d_blanked || nframes <= 0 || !framing_ok(clk.fmt, bytes) || clk.granularity < 1)
        return CS_ERR_ARG;
    CS_CUDA_TRY(cudaMemsetAsync(d_blanked, 0, sizeof(unsigned long long), st));
    k_vdif_ranges<<<blocks_for(nframes, 128), 128, 0, st>>>(framed, bytes, clk, nframes, ranges, d_blanked),
        cs_count_launches(1);
    return (int)cudaGetLastError();
}

int cs_framed_decode(const uint8_t* framed, int64_t bytes, const CsFraming& fmt, const int* d_offset,
                     const int2* ranges, int64_t nsamp, const float lut[4], float* out, unsigned long long* d_good,
                     cudaStream_t st)
{
    if (!framing_ok(fmt, bytes) || nsamp <= 0 || !out || !d_good || !ranges) return CS_ERR_ARG;
    CS_CUDA_TRY(cudaMemsetAsync(d_good, 0, sizeof(unsigned long long), st));
    k_decode_framed<<<blocks_for(nsamp, 256), 256, 0, st>>>(framed, bytes, fmt, d_offset, ranges, nsamp, lut[0],
                                                           lut[1], lut[2], lut[3], out, d_good),
        cs_count_launches(1);
    return (int)cudaGetLastError();
}

int cs_framed_deframe(const uint8_t* framed, int64_t bytes, const CsFraming& fmt, const int* d_offset,
                      const int2* ranges, int64_t nframes, uint8_t* payload, uint32_t* mask, cudaStream_t st)
{
    if (!framing_ok(fmt, bytes) || nframes <= 0 || !payload || !ranges) return CS_ERR_ARG;
    if ((uintptr_t)payload % 4 || ((uintptr_t)mask % 4)) return CS_ERR_ARG;
    const int64_t nwords = nframes * (fmt.payload_bytes / 4);
    k_deframe<<<blocks_for(nwords, 256), 256, 0, st>>>(framed, bytes, fmt, d_offset, nframes, (uint32_t*)payload),
        cs_count_launches(1);
    if (mask) {
        const int64_t nsamp = nframes * ((int64_t)fmt.payload_bytes * 4 / fmt.nch), mwords = (nsamp + 31) / 32;
        k_valid_mask<<<blocks_for(mwords, 256), 256, 0, st>>>(ranges, fmt, nframes, mwords, mask),
            cs_count_launches(1);
    }
    return (int)cudaGetLastError();
}

int cs_framed_planes(const uint8_t* framed, int64_t bytes, const CsFraming& fmt, const int* d_offset,
                     const int2* ranges, int64_t nframes, int64_t ngroups, uint32_t* planes, uint32_t* mask,
                     cudaStream_t st)
{
    if (!framing_ok(fmt, bytes) || ngroups <= 0 || !planes || !mask || !ranges) return CS_ERR_ARG;
    const unsigned nb = blocks_for(ngroups, 256);
#define CS_PLANES(N) \
    k_deframe_planes<N><<<nb, 256, 0, st>>>(framed, bytes, fmt, d_offset, ranges, nframes, ngroups, planes, mask)
    switch (fmt.nch) {
        case 1: CS_PLANES(1); break;
        case 4: CS_PLANES(4); break;
        case 8: CS_PLANES(8); break;
        case 16: CS_PLANES(16); break;
        default: return CS_ERR_ARG;
    }
#undef CS_PLANES
    cs_count_launches(1);
    return (int)cudaGetLastError();
}
