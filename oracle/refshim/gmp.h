/*
 * Minimal GMP compatibility header for compiling the reference CPU engine
 * here, where the GMP runtime (libgmp.so.10) is installed without its
 * development header.  It declares only the documented mpz API that the
 * reference uses, bound to the runtime's exported __gmpz_* entry points, and
 * the documented mpz_t layout.  Test infrastructure only.
 */
#ifndef CTD_REFSHIM_GMP_H
#define CTD_REFSHIM_GMP_H

#include <stddef.h>

#define __GNU_MP_VERSION 6
#define __GNU_MP_VERSION_MINOR 3
#define __GNU_MP_VERSION_PATCHLEVEL 0

#ifdef __cplusplus
extern "C" {
#endif

typedef unsigned long int mp_limb_t;
typedef unsigned long int mp_bitcnt_t;
typedef long int mp_size_t;

typedef struct {
    int _mp_alloc;
    int _mp_size;
    mp_limb_t *_mp_d;
} __mpz_struct;

typedef __mpz_struct mpz_t[1];
typedef __mpz_struct *mpz_ptr;
typedef const __mpz_struct *mpz_srcptr;

#define mpz_init __gmpz_init
#define mpz_clear __gmpz_clear
#define mpz_set __gmpz_set
#define mpz_swap __gmpz_swap
#define mpz_init_set_ui __gmpz_init_set_ui
#define mpz_init_set_str __gmpz_init_set_str
#define mpz_add __gmpz_add
#define mpz_add_ui __gmpz_add_ui
#define mpz_sub __gmpz_sub
#define mpz_sub_ui __gmpz_sub_ui
#define mpz_mul __gmpz_mul
#define mpz_mul_ui __gmpz_mul_ui
#define mpz_fdiv_q __gmpz_fdiv_q
#define mpz_fdiv_q_ui __gmpz_fdiv_q_ui
#define mpz_fdiv_qr __gmpz_fdiv_qr
#define mpz_fdiv_ui __gmpz_fdiv_ui
#define mpz_mul_2exp __gmpz_mul_2exp
#define mpz_pow_ui __gmpz_pow_ui
#define mpz_get_str __gmpz_get_str
#define mpz_cmp __gmpz_cmp
#define mpz_limbs_read __gmpz_limbs_read
#define mpz_sizeinbase __gmpz_sizeinbase

void mpz_init(mpz_ptr);
void mpz_clear(mpz_ptr);
void mpz_set(mpz_ptr, mpz_srcptr);
void mpz_swap(mpz_ptr, mpz_ptr);
void mpz_init_set_ui(mpz_ptr, unsigned long int);
int mpz_init_set_str(mpz_ptr, const char *, int);
void mpz_add(mpz_ptr, mpz_srcptr, mpz_srcptr);
void mpz_add_ui(mpz_ptr, mpz_srcptr, unsigned long int);
void mpz_sub(mpz_ptr, mpz_srcptr, mpz_srcptr);
void mpz_sub_ui(mpz_ptr, mpz_srcptr, unsigned long int);
void mpz_mul(mpz_ptr, mpz_srcptr, mpz_srcptr);
void mpz_mul_ui(mpz_ptr, mpz_srcptr, unsigned long int);
void mpz_fdiv_q(mpz_ptr, mpz_srcptr, mpz_srcptr);
unsigned long int mpz_fdiv_q_ui(mpz_ptr, mpz_srcptr, unsigned long int);
void mpz_fdiv_qr(mpz_ptr, mpz_ptr, mpz_srcptr, mpz_srcptr);
unsigned long int mpz_fdiv_ui(mpz_srcptr, unsigned long int);
void mpz_mul_2exp(mpz_ptr, mpz_srcptr, mp_bitcnt_t);
void mpz_pow_ui(mpz_ptr, mpz_srcptr, unsigned long int);
char *mpz_get_str(char *, int, mpz_srcptr);
int mpz_cmp(mpz_srcptr, mpz_srcptr);
const mp_limb_t *mpz_limbs_read(mpz_srcptr);
size_t mpz_sizeinbase(mpz_srcptr, int);

#ifdef __cplusplus
}
#endif

/* documented as macros in the GMP manual */
#define mpz_sgn(z) ((z)->_mp_size < 0 ? -1 : (z)->_mp_size > 0)
#define mpz_size(z) ((size_t)((z)->_mp_size < 0 ? -(z)->_mp_size : (z)->_mp_size))

#endif
