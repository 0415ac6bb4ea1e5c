/*
 * lss_oracle.c -- CPU oracle for the 2-D Heston/SABR ADI hot path.
 * TEST INFRASTRUCTURE ONLY (see lss_oracle.h): never linked into the product.
 *
 * Build (oracle/Makefile): gcc -O2 -ffp-contract=off -fPIC -shared.
 * -ffp-contract=off keeps a*b+c as two roundings, as the reference's MSVC/x86
 * build evaluates it, on every host (including aarch64, where gcc would
 * otherwise fuse into FMA).
 */
#include "lss_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define REAL double
#define SFX(name) name##_f64
#define ASINH asinh
#define SINH sinh
#define COSH cosh
#include "lss_oracle_impl.h"
#include "lss_oracle_1d_impl.h"
#undef REAL
#undef SFX
#undef ASINH
#undef SINH
#undef COSH

#define REAL float
#define SFX(name) name##_f32
#define ASINH asinhf
#define SINH sinhf
#define COSH coshf
#include "lss_oracle_impl.h"
#include "lss_oracle_1d_impl.h"
#undef REAL
#undef SFX
#undef ASINH
#undef SINH
#undef COSH

int lsso_coefficients_f64(const lsso_problem *p, double t, double *out)
{
    int rc = validate_f64(p);
    if (rc) return rc;
    ctx_f64 c;
    if (ctx_init_f64(&c, p)) return -1;
    fill_tables_f64(&c, t);
    const size_t n = (size_t)p->nx * p->ny;
    memcpy(out, c.M, sizeof(double) * n * 10);
    ctx_free_f64(&c);
    return 0;
}
