/* Declaration-only stand-in for <fftw3.h>.
 *
 * The reference's architecture.h / types_generic.h include <fftw3.h> to name
 * fftwf_plan and fftwf_complex and, in inline FFT wrappers that the oracle
 * never calls, a few FFTW entry points.  FFTW is not installed here, so this
 * header only declares those names; nothing defines them, and an accidental
 * call would fail to link, which is intended.
 */
#ifndef ORACLE_REFSHIM_FFTW3_H
#define ORACLE_REFSHIM_FFTW3_H
#ifdef __cplusplus
extern "C" {
#endif
typedef float fftwf_complex[2];
typedef struct fftwf_plan_opaque *fftwf_plan;
#define FFTW_FORWARD (-1)
#define FFTW_MEASURE (0U)
fftwf_plan fftwf_plan_dft_1d(int n, fftwf_complex* in, fftwf_complex* out, int sign, unsigned flags);
fftwf_plan fftwf_plan_dft_r2c_1d(int n, float* in, fftwf_complex* out, unsigned flags);
void fftwf_execute_dft(const fftwf_plan p, fftwf_complex* in, fftwf_complex* out);
void fftwf_execute_dft_r2c(const fftwf_plan p, float* in, fftwf_complex* out);
void fftwf_destroy_plan(fftwf_plan p);
#ifdef __cplusplus
}
#endif
#endif
