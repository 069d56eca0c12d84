/* Declarations of the GMP floating-point API used by the CPU port.
 *
 * Test infrastructure only.  The machines this runs on have the GMP runtime
 * (libgmp.so.10, a dependency of gcc) but no development headers, so the
 * handful of public entry points the port needs are declared here from GMP's
 * documented C ABI: mpf_t is an array of one struct {int _mp_prec;
 * int _mp_size; long _mp_exp; mp_limb_t *_mp_d;} and the documented mpf_*
 * names are exported with the __gmpf_ prefix (gmp_* printing with __gmp_).
 * GMP version pinned by the reference: 6.2.1 (external/gmp/Makefile.am:1);
 * runtime here 6.3.0 (same ABI, libgmp.so.10).
 */
#ifndef SDPG_GMP_ABI_H
#define SDPG_GMP_ABI_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef unsigned long mp_limb_t;
typedef long mp_exp_t;
typedef unsigned long mp_bitcnt_t;
typedef struct {
    int _mp_prec;
    int _mp_size;
    mp_exp_t _mp_exp;
    mp_limb_t *_mp_d;
} __mpf_struct;
typedef __mpf_struct mpf_t[1];
typedef __mpf_struct *mpf_ptr;
typedef const __mpf_struct *mpf_srcptr;

void __gmpf_set_default_prec(mp_bitcnt_t);
mp_bitcnt_t __gmpf_get_default_prec(void);
void __gmpf_init(mpf_ptr);
void __gmpf_init2(mpf_ptr, mp_bitcnt_t);
void __gmpf_clear(mpf_ptr);
void __gmpf_set(mpf_ptr, mpf_srcptr);
void __gmpf_set_d(mpf_ptr, double);
void __gmpf_set_si(mpf_ptr, long);
void __gmpf_set_ui(mpf_ptr, unsigned long);
int __gmpf_set_str(mpf_ptr, const char *, int);
double __gmpf_get_d(mpf_srcptr);
void __gmpf_add(mpf_ptr, mpf_srcptr, mpf_srcptr);
void __gmpf_sub(mpf_ptr, mpf_srcptr, mpf_srcptr);
void __gmpf_mul(mpf_ptr, mpf_srcptr, mpf_srcptr);
void __gmpf_div(mpf_ptr, mpf_srcptr, mpf_srcptr);
void __gmpf_sqrt(mpf_ptr, mpf_srcptr);
void __gmpf_neg(mpf_ptr, mpf_srcptr);
void __gmpf_abs(mpf_ptr, mpf_srcptr);
int __gmpf_cmp(mpf_srcptr, mpf_srcptr);
void __gmpf_mul_2exp(mpf_ptr, mpf_srcptr, mp_bitcnt_t);
void __gmpf_div_2exp(mpf_ptr, mpf_srcptr, mp_bitcnt_t);
int __gmp_snprintf(char *, size_t, const char *, ...);

#define mpf_set_default_prec __gmpf_set_default_prec
#define mpf_init __gmpf_init
#define mpf_init2 __gmpf_init2
#define mpf_clear __gmpf_clear
#define mpf_set __gmpf_set
#define mpf_set_d __gmpf_set_d
#define mpf_set_si __gmpf_set_si
#define mpf_set_ui __gmpf_set_ui
#define mpf_set_str __gmpf_set_str
#define mpf_get_d __gmpf_get_d
#define mpf_add __gmpf_add
#define mpf_sub __gmpf_sub
#define mpf_mul __gmpf_mul
#define mpf_div __gmpf_div
#define mpf_sqrt __gmpf_sqrt
#define mpf_neg __gmpf_neg
#define mpf_abs __gmpf_abs
#define mpf_cmp __gmpf_cmp
#define mpf_div_2exp __gmpf_div_2exp
#define gmp_snprintf __gmp_snprintf
#define mpf_sgn(F) ((F)->_mp_size < 0 ? -1 : (F)->_mp_size > 0)

#ifdef __cplusplus
}
#endif
#endif
