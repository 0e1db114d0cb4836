/* Exports the reference's GENERIC vector kernels (architecture.h, ARCH=4) as
 * plain C symbols so that the test suite can call the reference itself.
 *
 * Nothing here re-implements a kernel: every function forwards to the inline
 * function that architecture.h defines, compiled from the reference tree.
 * Built by oracle/Makefile into oracle/_ref/libref_generic.so.
 */
#include "architecture.h"

extern "C" {

/* architecture.h:405-421  acc[i] += a[i]*b[i] */
int ref_addproduct_32fc(fc32* a, fc32* b, fc32* acc, int n)
{ return genericAddProduct_32fc(a, b, acc, n); }

/* architecture.h:427-433  acc[i] += a[i]*conj(b[i]) */
int ref_addproduct_32fc_conj(fc32* a, fc32* b, fc32* acc, int n)
{ return genericAddProduct_32fc_conj(a, b, acc, n); }

/* architecture.h:440-456  a*=m, b*=m, acc += a*conj(b) */
int ref_addproduct_32fc_conjmul(fc32* a, fc32* b, fc32* m, fc32* acc, int n)
{ return genericAddProduct_32fc_conjMul(a, b, m, acc, n); }

/* architecture.h:462-474  a*=m, acc.re += |a|^2 */
int ref_addproduct_32fc_conjmul_self(fc32* a, fc32* m, fc32* acc, int n)
{ return genericAddProduct_cf32_conjMul_self(a, m, acc, n); }

/* architecture.h:270-278  dst = a*b */
int ref_mul_32fc(fc32* a, fc32* b, fc32* dst, int n)
{ return genericMul_32fc(a, b, dst, n); }

/* architecture.h:282-289  dst = a*conj(b) */
int ref_mul_32fc_conj(fc32* a, fc32* b, fc32* dst, int n)
{ return genericMul_32fc_conj(a, b, dst, n); }

/* architecture.h:492-500  interleaved {cos, sin} of each argument */
int ref_sincos_32f(f32* arg, f32* dst_sin_unused, f32* dst_cossin, int n)
{ return genericSinCos_32f(arg, dst_sin_unused, dst_cossin, n); }

}
