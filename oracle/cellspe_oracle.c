/* CPU oracle for the GB300 FX correlator / spectrometer hot path.
 * TEST INFRASTRUCTURE ONLY -- see cellspe_oracle.h for scope and pins.
 * Compiled with -ffp-contract=off so that FP32 products and sums are rounded
 * one operation at a time, as in the reference's scalar generic loops.
 */
#include "cellspe_oracle.h"
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ---------------------------------------------------------------------- */
/* 2-bit unpack                                                            */
/* ---------------------------------------------------------------------- */
static inline unsigned field2(const uint8_t* raw, int64_t fidx, int msb_first)
{
    uint8_t b = raw[fidx >> 2];
    int pos = (int)(fidx & 3);
    int shift = msb_first ? (6 - 2 * pos) : (2 * pos);
    return (b >> shift) & 3u;
}

void orc_unpack2bit(const uint8_t* raw, int64_t nsamp, int nchan, int msb_first,
                    const float lut[4], float* out)
{
    for (int c = 0; c < nchan; c++) {
        float* o = out + (int64_t)c * nsamp;
        for (int64_t t = 0; t < nsamp; t++)
            o[t] = lut[field2(raw, t * nchan + c, msb_first)];
    }
}

/* ---------------------------------------------------------------------- */
/* Framed Mark5B: first frame, fill-pattern blanking, decode               */
/* ---------------------------------------------------------------------- */
#define M5B_FRAME 10016
#define M5B_PAYLOAD 10000
#define M5B_FILL64 0x1122334411223344ULL
#define M5B_FILL32 0x11223344U

int orc_mark5b_find_first_frame(const uint8_t* d, int64_t bytes)
{
    if (bytes > (1 << 20)) bytes = 1 << 20;
    bytes -= M5B_FRAME + 4;
    for (int64_t i = 0; i < bytes; i++)
        if (d[i] == 0xED && d[i + 1] == 0xDE && d[i + 2] == 0xAD && d[i + 3] == 0xAB &&
            d[i + M5B_FRAME] == 0xED && d[i + M5B_FRAME + 1] == 0xDE && d[i + M5B_FRAME + 2] == 0xAD &&
            d[i + M5B_FRAME + 3] == 0xAB)
            return (int)i;
    return -1;
}

static uint64_t rd64(const uint8_t* p, int64_t i) { uint64_t v; memcpy(&v, p + 8 * i, 8); return v; }
static uint32_t rd32(const uint8_t* p, int64_t i) { uint32_t v; memcpy(&v, p + 4 * i, 4); return v; }

/* binary searches of blanker_mark5.c: boundary between data and fill words */
static int first_invalid(const uint8_t* p, int start, int end)
{
    int n = end - start, i = n / 2, r = n - 1;
    for (int s = n / 4; s > 0; s >>= 1) {
        if (rd64(p, start + i) == M5B_FILL64) { r = i; i -= s; }
        else i += s;
    }
    r = 8 * (start + r);
    if (rd32(p, r / 4 - 1) == M5B_FILL32) r -= 4;
    return r;
}

static int first_valid(const uint8_t* p, int start, int end)
{
    int n = end - start, i = n / 2, r = n - 1;
    for (int s = n / 4; s > 0; s >>= 1) {
        if (rd64(p, start + i) != M5B_FILL64) { r = i; i -= s; }
        else i += s;
    }
    r = 8 * (start + r);
    if (rd32(p, r / 4 - 2) == M5B_FILL32) r += 4;
    return r;
}

void orc_mark5b_valid_range(const uint8_t* p, int* start, int* end)
{
    const int nword = M5B_PAYLOAD / 8;
    int s_ok = rd64(p, 0) != M5B_FILL64, e_ok = rd64(p, nword - 1) != M5B_FILL64;
    if (s_ok && e_ok) { *start = 0; *end = 1 << 30; }
    else if (!s_ok && !e_ok) { *start = 1 << 30; *end = 0; }
    else if (s_ok) { *start = 0; *end = first_invalid(p, 0, nword); }
    else { *start = first_valid(p, 0, nword); *end = 1 << 30; }
}

int64_t orc_mark5b_decode_framed(const uint8_t* framed, int64_t bytes, int nchan, int64_t nsamp, float* out)
{
    static const float lut[4] = {-3.3359f, 1.0f, -1.0f, 3.3359f};
    int off = orc_mark5b_find_first_frame(framed, bytes);
    if (off < 0) return -1;
    const int bps = nchan / 4;                       /* bytes per sample time */
    const int spf = M5B_PAYLOAD / bps;
    int64_t good = 0;
    for (int64_t t = 0; t < nsamp; t++) {
        int64_t f = t / spf;
        int64_t fo = off + f * M5B_FRAME;
        const uint8_t* p = framed + fo + 16;
        int sv, ev;
        orc_mark5b_valid_range(p, &sv, &ev);
        int i = (int)(t % spf) * bps;
        int valid = i >= sv && i < ev;
        good += valid;
        for (int c = 0; c < nchan; c++) {
            unsigned code = (p[i + c / 4] >> (2 * (c % 4))) & 3u;
            out[(int64_t)c * nsamp + t] = valid ? lut[code] : 0.0f;
        }
        /* the decoder moves to the next frame as soon as a payload is used
         * up and fails when there is none (mark5_format_mark5b.c:1901-1908,
         * mark5_stream_memory.c:59-71), also after the last wanted sample */
        if (i + bps >= M5B_PAYLOAD && fo + 2 * M5B_FRAME > bytes) return -1;
    }
    return good;
}

/* ---------------------------------------------------------------------- */
/* Framed VDIF (mark5access format_vdif.c, blanker_mark5.c:282-316)         */
/* ---------------------------------------------------------------------- */
static uint32_t le32(const uint8_t* p)
{
    return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}

/* MJD of 1 January (even e) or 1 July (odd e) of year 2000 + e/2: the VDIF
 * reference epochs (format_vdif.c:145-155 tabulates them), from the civil
 * calendar: days since 1970-01-01 by the era/day-of-era method, + 40587. */
static int vdif_epoch_mjd(int e)
{
    int y = 2000 + e / 2, m = (e & 1) ? 7 : 1, d = 1;
    y -= m <= 2;
    const int era = y / 400, yoe = y - era * 400;
    const int doy = (153 * (m + (m > 2 ? -3 : 9)) + 2) / 5 + d - 1;
    const int doe = yoe * 365 + yoe / 4 - yoe / 100 + doy;
    return era * 146097 + doe - 719468 + 40587;
}

typedef struct {
    int hsize, databytes, framebytes;
    double framens;
    int fg, gframens;
    int mjd0, sec0, ns0;
} orc_vdif_stream;

/* mark5_stream_frame_time_vdif (format_vdif.c:135-200), leap seconds 0 */
static void vdif_frame_time(const uint8_t* h, double framens, int* mjd, int* sec, double* ns)
{
    const uint32_t w0 = le32(h), w1 = le32(h + 4);
    int seconds = (int)(w0 & 0x3FFFFFFF);
    int days = seconds / 86400;
    seconds -= days * 86400;
    *mjd = days + vdif_epoch_mjd((int)((w1 >> 24) & 0x3F));
    *sec = seconds;
    *ns = (double)(w1 & 0x00FFFFFF) * framens;
}

/* mark5_format_vdif_init (format_vdif.c:2121-2257) with the header-derived
 * payload size also used for the frame duration */
static int vdif_open(const uint8_t* d, int64_t bytes, int mbps, orc_vdif_stream* s)
{
    if (bytes < 32 || mbps <= 0) return -2;
    s->hsize = (d[3] & 0x40) ? 16 : 32;
    s->framebytes = (int)(le32(d + 8) & 0x00FFFFFF) * 8;
    s->databytes = s->framebytes - s->hsize;
    if (s->databytes < 8 || bytes < 2 * (int64_t)s->framebytes) return -2;
    const int num = s->databytes * 8 * 1000, den = mbps;
    s->framens = (double)num / (double)den;
    for (s->fg = 1; s->fg < 128; s->fg *= 2)
        if ((int)((unsigned)s->fg * (unsigned)num) % den == 0) break;
    if (s->fg >= 128) s->fg = 1;
    s->gframens = (int)(s->fg * s->framens + 0.5);
    double dns;
    vdif_frame_time(d, s->framens, &s->mjd0, &s->sec0, &dns);
    s->ns0 = (int)(dns + 0.5);
    return 0;
}

/* Payload offset of frame f.  The format name "VDIF_..." opens the stream
 * with 32-byte headers; on a legacy header mark5_format_vdif_init switches to
 * 16 bytes (format_vdif.c:2209-2220) after it has already pointed the first
 * payload 32 bytes into frame 0 (:2196), so frame 0 of a legacy stream is
 * read from byte 32 on (its last 16 bytes come from the next frame). */
static int vdif_payload_offset(const orc_vdif_stream* s, int64_t f)
{
    return f == 0 ? 32 : s->hsize;
}

static int vdif_ok(const uint8_t* framed, int64_t bytes, const orc_vdif_stream* s, int64_t f)
{
    if ((f + 1) * (int64_t)s->framebytes > bytes) return 0;
    const uint8_t* h = framed + f * (int64_t)s->framebytes;
    if (f > 0) {
        if (s->mjd0 && f % s->fg == 0) {
            int mjd_d, sec_d;
            double ns_d;
            vdif_frame_time(h, s->framens, &mjd_d, &sec_d, &ns_d);
            long long ns_t = f * (long long)(s->gframens / s->fg) + (long long)s->ns0;
            int sec_t = (int)(ns_t / 1000000000LL);
            ns_t -= (long long)sec_t * 1000000000LL;
            sec_t += s->sec0;
            int mjd_t = sec_t / 86400;
            sec_t -= mjd_t * 86400;
            mjd_t += s->mjd0;
            if (mjd_t != mjd_d || sec_t != sec_d || fabs((double)ns_t - ns_d) > 0.000001) return 0;
        }
        if ((le32(h) >> 31) & 1u) return 0;
    }
    const uint8_t* p = h + vdif_payload_offset(s, f);
    const int nword = s->databytes / 8;
    if (rd64(p, 0) == M5B_FILL64 || rd64(p, nword - 1) == M5B_FILL64) return 0;
    return 1;
}

int orc_vdif_first_time(const uint8_t* framed, int64_t bytes, int mbps, int* mjd, int* sec, int* ns)
{
    orc_vdif_stream s;
    if (vdif_open(framed, bytes, mbps, &s)) return -2;
    *mjd = s.mjd0;
    *sec = s.sec0;
    *ns = s.ns0;
    return 0;
}

int orc_vdif_frame_ok(const uint8_t* framed, int64_t bytes, int mbps, int64_t f)
{
    orc_vdif_stream s;
    if (vdif_open(framed, bytes, mbps, &s)) return -2;
    return vdif_ok(framed, bytes, &s, f);
}

int64_t orc_vdif_decode_framed(const uint8_t* framed, int64_t bytes, int nchan, int mbps, int64_t nsamp, float* out)
{
    static const float lut[4] = {-3.3359f, -1.0f, 1.0f, 3.3359f};
    if (!(nchan == 1 || nchan == 2 || nchan == 4 || nchan == 8 || nchan == 16)) return -2;
    orc_vdif_stream s;
    if (vdif_open(framed, bytes, mbps, &s)) return -2;
    if (nchan < 4 && nsamp % (4 / nchan)) return -3;
    if ((s.databytes * 4) % nchan) return -2;
    const int64_t spf = (int64_t)s.databytes * 4 / nchan;
    int64_t good = 0, fcur = -1;
    int ok = 0;
    for (int64_t t = 0; t < nsamp; t++) {
        const int64_t f = t / spf, st = t % spf;
        if (f != fcur) { fcur = f; ok = vdif_ok(framed, bytes, &s, f); }
        const uint8_t* p = framed + f * (int64_t)s.framebytes + vdif_payload_offset(&s, f);
        good += ok;
        for (int c = 0; c < nchan; c++) {
            const int64_t bit = (st * nchan + c) * 2;
            const unsigned code = (p[bit >> 3] >> (bit & 7)) & 3u;
            out[(int64_t)c * nsamp + t] = ok ? lut[code] : 0.0f;
        }
        /* next frame as soon as a payload is used up (format_vdif.c:684-692) */
        if (st == spf - 1 && (f + 2) * (int64_t)s.framebytes > bytes) return -1;
    }
    return good;
}

/* ---------------------------------------------------------------------- */
/* Generic complex MAC (architecture.h:405-433)                            */
/* ---------------------------------------------------------------------- */
void orc_addproduct_32fc(const orc_cf32* a, const orc_cf32* b, orc_cf32* acc, int n)
{
    for (int i = 0; i < n; i++) {
        acc[i].re += (a[i].re * b[i].re) - (a[i].im * b[i].im);
        acc[i].im += (a[i].im * b[i].re) + (a[i].re * b[i].im);
    }
}

void orc_addproduct_32fc_conj(const orc_cf32* a, const orc_cf32* b, orc_cf32* acc, int n)
{
    for (int i = 0; i < n; i++) {
        acc[i].re += (a[i].re * b[i].re) + (a[i].im * b[i].im);
        acc[i].im += (a[i].im * b[i].re) - (a[i].re * b[i].im);
    }
}

/* ---------------------------------------------------------------------- */
/* FFTs                                                                    */
/* ---------------------------------------------------------------------- */
static int ilog2(int n) { int l = 0; while ((1 << l) < n) l++; return l; }

static unsigned bitrev(unsigned x, int bits)
{
    unsigned r = 0;
    for (int i = 0; i < bits; i++) { r = (r << 1) | (x & 1u); x >>= 1; }
    return r;
}

void orc_cfft_f32(const orc_cf32* in, orc_cf32* out, int n)
{
    int lg = ilog2(n);
    orc_cf32* tmp = (orc_cf32*)malloc(sizeof(orc_cf32) * (size_t)n);
    for (int i = 0; i < n; i++) tmp[bitrev((unsigned)i, lg)] = in[i];
    for (int len = 2; len <= n; len <<= 1) {
        int half = len >> 1;
        for (int j = 0; j < half; j++) {
            double ang = -2.0 * M_PI * (double)j / (double)len;
            float wr = (float)cos(ang), wi = (float)sin(ang);
            for (int i = 0; i < n; i += len) {
                orc_cf32 u = tmp[i + j], v = tmp[i + j + half];
                float tr = v.re * wr - v.im * wi;
                float ti = v.re * wi + v.im * wr;
                tmp[i + j].re = u.re + tr;          tmp[i + j].im = u.im + ti;
                tmp[i + j + half].re = u.re - tr;   tmp[i + j + half].im = u.im - ti;
            }
        }
    }
    memcpy(out, tmp, sizeof(orc_cf32) * (size_t)n);
    free(tmp);
}

void orc_cfft_f64(const double* in, double* out, int n)
{
    int lg = ilog2(n);
    double* t = (double*)malloc(sizeof(double) * 2 * (size_t)n);
    for (int i = 0; i < n; i++) {
        unsigned r = bitrev((unsigned)i, lg);
        t[2 * r] = in[2 * i]; t[2 * r + 1] = in[2 * i + 1];
    }
    for (int len = 2; len <= n; len <<= 1) {
        int half = len >> 1;
        for (int j = 0; j < half; j++) {
            double ang = -2.0 * M_PI * (double)j / (double)len;
            double wr = cos(ang), wi = sin(ang);
            for (int i = 0; i < n; i += len) {
                double* u = t + 2 * (i + j);
                double* v = t + 2 * (i + j + half);
                double tr = v[0] * wr - v[1] * wi, ti = v[0] * wi + v[1] * wr;
                v[0] = u[0] - tr; v[1] = u[1] - ti;
                u[0] = u[0] + tr; u[1] = u[1] + ti;
            }
        }
    }
    memcpy(out, t, sizeof(double) * 2 * (size_t)n);
    free(t);
}

void orc_rfft_f32(const float* in, orc_cf32* out, int n)
{
    int m = n / 2;
    orc_cf32* z = (orc_cf32*)malloc(sizeof(orc_cf32) * (size_t)m);
    orc_cf32* Z = (orc_cf32*)malloc(sizeof(orc_cf32) * (size_t)m);
    for (int i = 0; i < m; i++) { z[i].re = in[2 * i]; z[i].im = in[2 * i + 1]; }
    orc_cfft_f32(z, Z, m);
    for (int k = 0; k <= m; k++) {
        orc_cf32 a = Z[k % m], b = Z[(m - k) % m];
        /* E = (a + conj b)/2,  O = (a - conj b)/(2i) */
        float er = 0.5f * (a.re + b.re), ei = 0.5f * (a.im - b.im);
        float orr = 0.5f * (a.im + b.im), oi = -0.5f * (a.re - b.re);
        double ang = -2.0 * M_PI * (double)k / (double)n;
        float wr = (float)cos(ang), wi = (float)sin(ang);
        out[k].re = er + (orr * wr - oi * wi);
        out[k].im = ei + (orr * wi + oi * wr);
    }
    out[0].im = 0.0f;
    out[m].im = 0.0f;
    free(z); free(Z);
}

/* ---------------------------------------------------------------------- */
/* Spectrometer (TaskCoreIPP::doMaths, one source)                         */
/* ---------------------------------------------------------------------- */
int orc_spec_overlapped_ffts(const orc_spec_cfg* cfg)
{
    return cfg->overlap * cfg->ffts_per_spectrum - (cfg->overlap - 1);
}

/* TaskCoreIPP::generate_windowfunction (TaskCoreIPP.cpp:569-605): None,
 * Cosine, Cosine2 as its loops; Hamming, Hann and Blackman (alpha 0.5) are
 * IPP's ippsWin*_32f_I, restated from IPP's published definitions with
 * x = 2 pi i / (n - 1) (IPP is absent: these three are not pinned). */
void orc_spec_window(int type, int n, float* w)
{
    for (int i = 0; i < n; i++) {
        if (type == 1 || type == 2) {
            double arg = M_PI * ((double)(float)i - 0.5 * (double)(float)n + 0.5) / (double)(float)n;
            double c = cos(arg);
            w[i] = (type == 1) ? (float)c : (float)(c * c);
            continue;
        }
        double x = 2.0 * M_PI * (double)i / (double)(n - 1);
        if (type == 3) w[i] = (float)(0.54 - 0.46 * cos(x));
        else if (type == 4) w[i] = (float)(0.5 - 0.5 * cos(x));
        else if (type == 5) w[i] = (float)(0.75 - 0.5 * cos(x) - 0.25 * cos(2.0 * x));
        else w[i] = 1.0f;
    }
}

static void pcal_fold(const float* x, int n, const orc_spec_cfg* cfg, const orc_cf32* rot,
                      orc_cf32* bins)
{
    int L = cfg->pcal_rotatorlen, T = cfg->pcal_tonebins;
    for (int s = 0; s + L <= n; s += L) {
        for (int i = 0; i < L; i++) {
            float re = x[s + i] * rot[i].re;   /* ippsMul_32f32fc */
            float im = x[s + i] * rot[i].im;
            bins[i % T].re += re;              /* ippsAdd_32fc_I fold */
            bins[i % T].im += im;
        }
    }
}

int orc_spectrometer(const float* samples, int64_t nsamp, const orc_spec_cfg* cfg,
                     float* power, orc_cf32* pcal_bins)
{
    const int N = cfg->fft_points, nb = N / 2 + 1;
    const int hop = N / cfg->overlap;
    const int novl = orc_spec_overlapped_ffts(cfg);
    const float scale = (float)(1.0 / (double)novl);
    float* w = (float*)malloc(sizeof(float) * (size_t)N);
    float* xw = (float*)malloc(sizeof(float) * (size_t)N);
    orc_cf32* X = (orc_cf32*)malloc(sizeof(orc_cf32) * (size_t)nb);
    orc_cf32* rot = NULL;
    orc_spec_window(cfg->window, N, w);
    if (cfg->pcal_tonebins > 0) {
        rot = (orc_cf32*)malloc(sizeof(orc_cf32) * (size_t)cfg->pcal_rotatorlen);
        double dphi = 2 * M_PI * (-cfg->pcal_offset_hz / cfg->sample_rate_hz);
        for (int i = 0; i < cfg->pcal_rotatorlen; i++) {
            rot[i].re = (float)cos(dphi * (double)i);
            rot[i].im = (float)sin(dphi * (double)i);
        }
    }
    int64_t pos = 0, remaining = nsamp;
    int acc = 0, spec = 0, curr = 0;
    float* P = power;
    orc_cf32* PC = pcal_bins;
    memset(P, 0, sizeof(float) * (size_t)nb);
    if (PC) memset(PC, 0, sizeof(orc_cf32) * (size_t)cfg->pcal_tonebins);
    while (remaining >= N) {
        const float* x = samples + pos;
        pos += hop;
        if (rot && PC && (curr % cfg->overlap) == 0) pcal_fold(x, N, cfg, rot, PC);
        for (int i = 0; i < N; i++) xw[i] = w[i] * x[i];
        orc_rfft_f32(xw, X, N);
        curr++;
        float re0 = X[0].re, reN2 = X[N / 2].re;
        float acc0 = P[0] + re0 * re0;
        float accN = P[nb - 1] + reN2 * reN2;
        for (int k = 1; k < nb - 1; k++) {
            float pw = X[k].re * X[k].re + X[k].im * X[k].im;
            P[k] += pw;
        }
        P[0] = acc0; P[nb - 1] = accN;
        remaining -= hop;
        if (++acc >= novl) {
            for (int k = 0; k < nb; k++) P[k] *= scale;
            spec++; acc = 0;
            pos += N - hop; remaining -= N - hop;
            P += nb;
            if (PC) PC += cfg->pcal_tonebins;
            if (remaining >= N) {
                memset(P, 0, sizeof(float) * (size_t)nb);
                if (PC) memset(PC, 0, sizeof(orc_cf32) * (size_t)cfg->pcal_tonebins);
            }
        }
    }
    free(w); free(xw); free(X); free(rot);
    return spec;
}

/* Two sources and their cross spectrum: TaskCoreIPP::doMaths with
 * num_sources = 2, num_xpols = 1 (TaskCoreIPP.cpp:394-513).  Per hop, each
 * source in turn: phase-cal fold when the FFT count (starting at 0 once,
 * advanced after every source's FFT) is a multiple of the overlap
 * (:414-418, :434-435), window, real FFT, auto power with DC/Nyquist as real
 * products (:437-447); then the cross spectrum X0 conj(X1) for bins
 * 1..N/2-1 through ippsConj + ippsAddProduct, with DC and Nyquist as real
 * products and zero imaginary parts (:456-487).  Spectra are scaled by
 * 1/core_overlapped_ffts (:491-499). */
int orc_spectrometer_xpol(const float* s0, const float* s1, int64_t nsamp, const orc_spec_cfg* cfg,
                          float* power, orc_cf32* xpol, orc_cf32* pcal_bins)
{
    const int N = cfg->fft_points, nb = N / 2 + 1;
    const int hop = N / cfg->overlap;
    const int novl = orc_spec_overlapped_ffts(cfg);
    const float scale = (float)(1.0 / (double)novl);
    const int nspec_max = (int)(nsamp / ((int64_t)N * cfg->ffts_per_spectrum));
    float* w = (float*)malloc(sizeof(float) * (size_t)N);
    float* xw = (float*)malloc(sizeof(float) * (size_t)N);
    orc_cf32* X[2];
    X[0] = (orc_cf32*)malloc(sizeof(orc_cf32) * (size_t)nb);
    X[1] = (orc_cf32*)malloc(sizeof(orc_cf32) * (size_t)nb);
    orc_cf32* conj1 = (orc_cf32*)malloc(sizeof(orc_cf32) * (size_t)nb);
    orc_cf32* rot = NULL;
    orc_spec_window(cfg->window, N, w);
    if (cfg->pcal_tonebins > 0) {
        rot = (orc_cf32*)malloc(sizeof(orc_cf32) * (size_t)cfg->pcal_rotatorlen);
        double dphi = 2 * M_PI * (-cfg->pcal_offset_hz / cfg->sample_rate_hz);
        for (int i = 0; i < cfg->pcal_rotatorlen; i++) {
            rot[i].re = (float)cos(dphi * (double)i);
            rot[i].im = (float)sin(dphi * (double)i);
        }
    }
    const size_t psz = (size_t)nspec_max * nb, tsz = (size_t)nspec_max * (size_t)cfg->pcal_tonebins;
    memset(power, 0, sizeof(float) * 2 * psz);
    memset(xpol, 0, sizeof(orc_cf32) * psz);
    if (pcal_bins && rot) memset(pcal_bins, 0, sizeof(orc_cf32) * 2 * tsz);
    int64_t pos = 0, remaining = nsamp;
    int acc = 0, spec = 0, curr = 0;
    while (remaining >= N && spec < nspec_max) {
        for (int rs = 0; rs < 2; rs++) {
            const float* x = (rs ? s1 : s0) + pos;
            float* P = power + (size_t)rs * psz + (size_t)spec * nb;
            if (rot && pcal_bins && (curr % cfg->overlap) == 0)
                pcal_fold(x, N, cfg, rot, pcal_bins + (size_t)rs * tsz + (size_t)spec * cfg->pcal_tonebins);
            for (int i = 0; i < N; i++) xw[i] = w[i] * x[i];
            orc_rfft_f32(xw, X[rs], N);
            curr++;
            float re0 = X[rs][0].re, reN2 = X[rs][N / 2].re;
            float acc0 = P[0] + re0 * re0;
            float accN = P[nb - 1] + reN2 * reN2;
            for (int k = 1; k < nb - 1; k++) P[k] += X[rs][k].re * X[rs][k].re + X[rs][k].im * X[rs][k].im;
            P[0] = acc0; P[nb - 1] = accN;
        }
        orc_cf32* XP = xpol + (size_t)spec * nb;
        float old0 = XP[0].re, oldN = XP[nb - 1].re;
        for (int k = 1; k < nb - 1; k++) { conj1[k].re = X[1][k].re; conj1[k].im = -X[1][k].im; }
        orc_addproduct_32fc(X[0] + 1, conj1 + 1, XP + 1, nb - 2);
        XP[0].re = old0 + X[0][0].re * X[1][0].re;
        XP[0].im = 0.0f;
        XP[nb - 1].re = oldN + X[0][N / 2].re * X[1][N / 2].re;
        XP[nb - 1].im = 0.0f;
        pos += hop;
        remaining -= hop;
        if (++acc >= novl) {
            float* P0 = power + (size_t)spec * nb;
            float* P1 = power + psz + (size_t)spec * nb;
            for (int k = 0; k < nb; k++) {
                P0[k] *= scale;
                P1[k] *= scale;
                XP[k].re *= scale;
                XP[k].im *= scale;
            }
            spec++; acc = 0;
            pos += N - hop; remaining -= N - hop;
        }
    }
    free(w); free(xw); free(X[0]); free(X[1]); free(conj1); free(rot);
    return spec;
}

void orc_pcal_tones(const orc_cf32* bins, int nbins, int ntones, orc_cf32* tones)
{
    for (int k = 0; k < ntones; k++) {
        double re = 0, im = 0;
        for (int n = 0; n < nbins; n++) {
            double a = -2.0 * M_PI * (double)((int64_t)k * n % nbins) / (double)nbins;
            re += bins[n].re * cos(a) - bins[n].im * sin(a);
            im += bins[n].re * sin(a) + bins[n].im * cos(a);
        }
        tones[k].re = (float)(re / nbins);
        tones[k].im = (float)(im / nbins);
    }
}

/* ---------------------------------------------------------------------- */
/* FX correlator, FP32 CPU path                                            */
/* ---------------------------------------------------------------------- */
typedef struct {
    const uint8_t* raw; int64_t bpi; int S, N, K; int64_t start;
    const int32_t* shift; const orc_cf32* phasor; const float* lut; int msb;
    orc_cf32* spectra; orc_cf32* vis;
    int t0, t1;            /* work range (units depend on the phase) */
} fx_job;

static void fstage_one(const fx_job* j, int s, int k, float* x, orc_cf32* X)
{
    const int N = j->N, C = N / 2;
    int64_t st = j->start + (int64_t)k * N + (j->shift ? j->shift[(int64_t)s * j->K + k] : 0);
    const uint8_t* r = j->raw + (int64_t)s * j->bpi;
    for (int n = 0; n < N; n++) x[n] = j->lut[field2(r, st + n, j->msb)];
    orc_rfft_f32(x, X, N);
    orc_cf32* o = j->spectra + ((int64_t)s * j->K + k) * C;
    if (j->phasor) {
        const orc_cf32* ph = j->phasor + ((int64_t)s * j->K + k) * C;
        for (int c = 0; c < C; c++) {       /* genericMul_32fc, architecture.h:270-278 */
            o[c].re = (X[c].re * ph[c].re) - (X[c].im * ph[c].im);
            o[c].im = (X[c].im * ph[c].re) + (X[c].re * ph[c].im);
        }
    } else {
        memcpy(o, X, sizeof(orc_cf32) * (size_t)C);
    }
}

static void* fstage_worker(void* arg)
{
    fx_job* j = (fx_job*)arg;
    float* x = (float*)malloc(sizeof(float) * (size_t)j->N);
    orc_cf32* X = (orc_cf32*)malloc(sizeof(orc_cf32) * (size_t)(j->N / 2 + 1));
    for (int u = j->t0; u < j->t1; u++) fstage_one(j, u / j->K, u % j->K, x, X);
    free(x); free(X);
    return NULL;
}

static void* xstage_worker(void* arg)
{
    fx_job* j = (fx_job*)arg;
    const int C = j->N / 2;
    for (int p = j->t0; p < j->t1; p++) {
        int i = (int)((sqrt(8.0 * p + 1.0) - 1.0) / 2.0);
        while ((i + 1) * (i + 2) / 2 <= p) i++;
        while (i * (i + 1) / 2 > p) i--;
        int jj = p - i * (i + 1) / 2;
        orc_cf32* acc = j->vis + (int64_t)p * C;
        for (int k = 0; k < j->K; k++)
            orc_addproduct_32fc_conj(j->spectra + ((int64_t)i * j->K + k) * C,
                                     j->spectra + ((int64_t)jj * j->K + k) * C, acc, C);
    }
    return NULL;
}

static void run_parallel(fx_job* base, int units, int nthreads, void* (*fn)(void*))
{
    if (nthreads < 1) nthreads = 1;
    if (nthreads > units) nthreads = units > 0 ? units : 1;
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nthreads);
    fx_job* jobs = (fx_job*)malloc(sizeof(fx_job) * (size_t)nthreads);
    for (int t = 0; t < nthreads; t++) {
        jobs[t] = *base;
        jobs[t].t0 = (int)((int64_t)units * t / nthreads);
        jobs[t].t1 = (int)((int64_t)units * (t + 1) / nthreads);
        if (nthreads == 1) fn(&jobs[t]);
        else pthread_create(&th[t], NULL, fn, &jobs[t]);
    }
    if (nthreads > 1)
        for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    free(th); free(jobs);
}

void orc_fx_fstage_fp32(const uint8_t* raw, int64_t bytes_per_input, int S, int N, int K,
                        int64_t start_sample, const int32_t* shift, const orc_cf32* phasor,
                        const float lut[4], int msb_first, orc_cf32* spectra, int nthreads)
{
    fx_job j = { raw, bytes_per_input, S, N, K, start_sample, shift, phasor, lut, msb_first,
                 spectra, NULL, 0, 0 };
    run_parallel(&j, S * K, nthreads, fstage_worker);
}

void orc_fx_fp32(const uint8_t* raw, int64_t bytes_per_input, int S, int N, int K,
                 int64_t start_sample, const int32_t* shift, const orc_cf32* phasor,
                 const float lut[4], int msb_first, orc_cf32* vis, int nthreads)
{
    const int C = N / 2;
    orc_cf32* spectra = (orc_cf32*)malloc(sizeof(orc_cf32) * (size_t)S * K * C);
    orc_fx_fstage_fp32(raw, bytes_per_input, S, N, K, start_sample, shift, phasor, lut,
                       msb_first, spectra, nthreads);
    fx_job j = { raw, bytes_per_input, S, N, K, start_sample, shift, phasor, lut, msb_first,
                 spectra, vis, 0, 0 };
    run_parallel(&j, S * (S + 1) / 2, nthreads, xstage_worker);
    free(spectra);
}
