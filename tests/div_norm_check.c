/* Exhaustive check of the block-matching kernel's division by the patch
 * norm (div_norm in vbm3d_gb300/csrc/bm2_impl.cuh): for each divisor b on
 * the command line, over every float a in [2^-100, FLT_MAX], compares
 * q + (a - q b) rcp (q = a * rcp, rcp = 1 / b, the remainder by one FMA, each
 * operation rounded once as the kernel's __fmul_rn / __fmaf_rn are) with
 * the IEEE quotient a / b.  Prints "b mismatches" per divisor.  Test
 * infrastructure (tests/test_div_norm.py). */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static float asf(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static uint32_t asu(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }

int main(int argc, char **argv)
{
    const uint32_t lo = asu(0x1p-100f), hi = 0x7f7fffffu; /* FLT_MAX */
    for (int k = 1; k < argc; k++) {
        const float b = strtof(argv[k], NULL);
        const float rcp = 1.0f / b;
        long long bad = 0;
#pragma omp parallel for reduction(+ : bad) schedule(static, 1 << 20)
        for (long long i = lo; i <= (long long)hi; i++) {
            const float a = asf((uint32_t)i);
            const float q = a * rcp;
            const float r = fmaf(-q, b, a);
            const float got = fmaf(r, rcp, q);
            if (asu(got) != asu(a / b)) bad++;
        }
        printf("%g %lld\n", b, bad);
    }
    return 0;
}
