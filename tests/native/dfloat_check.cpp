/* Checks the double-float arithmetic of the exact denoise rounding
 * (libcraw_gb300/csrc/kernels/dfloat.cuh) against long double on the host:
 * prints the largest relative error of each operation over a seeded sweep.
 * Built and run by tests/test_dfloat.py with -ffp-contract=off. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "../../libcraw_gb300/csrc/kernels/dfloat.cuh"

typedef long double LD;

static LD val(dfl a) { return (LD)a.hi + (LD)a.lo; }

static dfl split(LD v)
{
    float hi = (float)v;
    float lo = (float)(v - (LD)hi);
    return df_make(hi, lo);
}

static uint64_t st = 0x9e3779b97f4a7c15ull;
static double uni(void)
{
    st ^= st << 13;
    st ^= st >> 7;
    st ^= st << 17;
    return (double)(st >> 11) * (1.0 / 9007199254740992.0);
}

static LD relerr(LD got, LD want)
{
    LD d = fabsl(got - want);
    return want != 0 ? d / fabsl(want) : d;
}

int main(int argc, char **argv)
{
    int n = argc > 1 ? atoi(argv[1]) : 200000;
    LD e_exp = 0, e_sqrt = 0, e_div = 0, e_mul = 0, e_add = 0, e_sub = 0;
    int rint_bad = 0;
    for (int i = 0; i < n; i++) {
        dfl yd = split((LD)uni() * 60.0L);
        e_exp = fmaxl(e_exp, relerr(val(df_exp_neg(yd)), expl(-val(yd))));

        LD a = (LD)uni() * 4000.0L + 1e-3L, b = (LD)uni() * 70.0L + 1e-3L;
        dfl ad = split(a), bd = split(b);
        e_sqrt = fmaxl(e_sqrt, relerr(val(df_sqrt(ad)), sqrtl(val(ad))));
        e_div = fmaxl(e_div, relerr(val(df_div(ad, bd)), val(ad) / val(bd)));
        e_mul = fmaxl(e_mul, relerr(val(df_mul(ad, bd)), val(ad) * val(bd)));
        e_add = fmaxl(e_add, relerr(val(df_add(ad, bd)), val(ad) + val(bd)));
        /* Differences of close values: error relative to the operands. */
        dfl cd = split(a + ((LD)uni() - 0.5L) * 1e-3L);
        e_sub = fmaxl(e_sub, fabsl(val(df_sub(ad, cd)) - (val(ad) - val(cd))) / fabsl(val(ad)));

        /* rint near half-integers. */
        dfl xd = split(floorl((LD)uni() * 4000.0L) + 0.5L + ((LD)uni() - 0.5L) * 1e-9L);
        if ((LD)df_rint(xd) != rintl(val(xd)))
            rint_bad++;
    }
    printf("exp %.3Le\nsqrt %.3Le\ndiv %.3Le\nmul %.3Le\nadd %.3Le\nsub %.3Le\nrint_bad %d\n", e_exp, e_sqrt,
           e_div, e_mul, e_add, e_sub, rint_bad);
    return 0;
}
