/* Thin C entry points over the reference's vendored mark5access 1.4.3 so the
 * test suite can decode a byte buffer with the library's own code path:
 * new_mark5_stream(new_mark5_stream_unpacker(1), <format string>) followed by
 * mark5_unpack() (mark5access/mark5_stream_unpacker.c).  Built by
 * oracle/Makefile into oracle/_ref/libref_mark5.so together with the
 * mark5access sources, which are compiled in place from the reference tree.
 */
#include <stdlib.h>
#include "mark5access/mark5_stream.h"

/* Decodes nsamp samples per channel of a headerless (payload-only) stream in
 * the given format ("Mark5B-512-16-2" ...).  out is nchan*nsamp floats,
 * channel-major.  Returns the number of good samples from mark5_unpack, or a
 * negative value when the format is not recognised. */
int ref_mark5_unpack(const char* format, const void* packed, int nsamp,
                     float* out, int* nchan_out)
{
    struct mark5_format_generic* f = new_mark5_format_generic_from_string(format);
    if (!f) return -1;
    struct mark5_stream* ms = new_mark5_stream(new_mark5_stream_unpacker(1), f);
    if (!ms) return -2;
    int nchan = ms->nchan;
    float** planes = (float**)malloc(sizeof(float*) * nchan);
    for (int c = 0; c < nchan; c++) planes[c] = out + (size_t)c * nsamp;
    int rc = mark5_unpack(ms, (void*)packed, planes, nsamp);
    if (nchan_out) *nchan_out = nchan;
    free(planes);
    delete_mark5_stream(ms);
    return rc;
}

/* Number of channels and bits per sample for a format string. */
int ref_mark5_format_info(const char* format, int* nchan, int* nbit)
{
    struct mark5_format_generic* f = new_mark5_format_generic_from_string(format);
    if (!f) return -1;
    struct mark5_stream* ms = new_mark5_stream(new_mark5_stream_unpacker(1), f);
    if (!ms) return -2;
    *nchan = ms->nchan;
    *nbit = ms->nbit;
    delete_mark5_stream(ms);
    return 0;
}

/* Decodes nsamp samples per channel of a framed stream (headers included)
 * through new_mark5_stream_memory() + mark5_stream_decode() -- the library's
 * framed path with its fill-pattern blanking (blanker_mark5.c).  Returns the
 * number of good (unblanked) samples, or a negative value on failure. */
int ref_mark5_decode_memory(const char* format, void* data, unsigned int bytes, int nsamp,
                            float* out, int* nchan_out, int* frameoffset_out)
{
    struct mark5_format_generic* f = new_mark5_format_generic_from_string(format);
    if (!f) return -1;
    struct mark5_stream* ms = new_mark5_stream(new_mark5_stream_memory(data, bytes), f);
    if (!ms) return -2;
    int nchan = ms->nchan;
    float** planes = (float**)malloc(sizeof(float*) * nchan);
    for (int c = 0; c < nchan; c++) planes[c] = out + (size_t)c * nsamp;
    if (nchan_out) *nchan_out = nchan;
    if (frameoffset_out) *frameoffset_out = ms->frameoffset;
    int rc = mark5_stream_decode(ms, nsamp, planes);
    free(planes);
    delete_mark5_stream(ms);
    return rc;
}

/* Time of the first frame as the library reads it when it opens a memory
 * stream (ms->mjd, ms->sec, ms->ns after mark5_format_init).  Returns 0, or a
 * negative value when the stream does not open. */
int ref_mark5_stream_time(const char* format, void* data, unsigned int bytes, int* mjd, int* sec, int* ns)
{
    struct mark5_format_generic* f = new_mark5_format_generic_from_string(format);
    if (!f) return -1;
    struct mark5_stream* ms = new_mark5_stream(new_mark5_stream_memory(data, bytes), f);
    if (!ms) return -2;
    *mjd = ms->mjd;
    *sec = ms->sec;
    *ns = ms->ns;
    delete_mark5_stream(ms);
    return 0;
}
