/* Host check of the float-pair bounded sum (the algorithm of df32.cuh's
 * bound_add / sigma_of / dfs_mul / dfs_fma, restated in C with the C library's
 * correctly rounded fmaf): on random stencil sums of float pairs it verifies
 *   - every partial sum of the extracted high parts (tau) is exact in a float,
 *   - the final pair (after one TwoSum) is within n^2 2^-46 B of the exact
 *     sum, B = sum |ch_k| |xh_k|  (the bound the design states),
 * against sums in binary128.  Prints the largest error / B seen and exits
 * non-zero on a violation.
 *
 * Usage: bounded_sum_check <trials> <seed>
 * Build: gcc -O2 -ffp-contract=off bounded_sum_check.c -lm
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* a binary128 type: long double on AArch64, __float128 on x86-64 */
#if defined(__aarch64__)
typedef long double quad;
#else
typedef __float128 quad;
#endif

static uint64_t rng_state;
static uint64_t next_u64(void) { /* SplitMix64 */
    uint64_t z = (rng_state += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static double uniform(void) { return (double)(next_u64() >> 11) * (1.0 / 9007199254740992.0); }

static float f_of_bits(uint32_t b) { float f; memcpy(&f, &b, 4); return f; }
static uint32_t bits_of_f(float f) { uint32_t b; memcpy(&b, &f, 4); return b; }

/* a double split into a float pair (hi, lo) with |lo| <= ulp(hi) / 2 */
static void split(double x, float *h, float *l) {
    *h = (float)x;
    *l = (float)(x - (double)*h);
}

static float sigma_of(float b) {
    /* __fmul_ru(b, 1 + 2^-16): round up by hand -- b * (1 + 2^-16) is exact in double */
    const double prod = (double)b * (1.0 + ldexp(1.0, -16));
    float bb = (float)prod;
    if ((double)bb < prod) bb = nextafterf(bb, INFINITY);
    int e = (int)(bits_of_f(bb) & 0x7f800000u);
    if (e > (253 << 23)) e = 253 << 23;
    return f_of_bits((uint32_t)(e + (1 << 23)));
}

int main(int argc, char **argv) {
    const long trials = argc > 1 ? atol(argv[1]) : 200000;
    rng_state = argc > 2 ? strtoull(argv[2], 0, 10) : 1;
    const int sizes[] = {3, 5, 7, 9, 13, 19};
    double worst[6] = {0};
    long bad = 0;
    for (long t = 0; t < trials; ++t) {
        const int si = (int)(t % 6), n = sizes[si];
        float ch[19], cl[19], xh[19], xl[19];
        /* coefficients: positive or mixed signs, magnitudes spread over 2^-8..1;
           values: one sign or mixed, magnitudes spread over up to 2^40 */
        const int mixed_c = (t / 6) % 2, mixed_x = (t / 12) % 2, spread = (int)((t / 24) % 4) * 13;
        for (int k = 0; k < n; ++k) {
            double c = ldexp(0.5 + uniform(), -(int)(uniform() * 8));
            if (mixed_c && uniform() < 0.5) c = -c;
            double x = ldexp(0.5 + uniform(), -(int)(uniform() * spread)) * ldexp(1.0, (int)(uniform() * 40) - 20);
            if (mixed_x && uniform() < 0.5) x = -x;
            split(c, &ch[k], &cl[k]);
            split(x, &xh[k], &xl[k]);
        }
        /* the bound and sigma */
        float b = 0.0f;
        for (int k = 0; k < n; ++k) b = fmaf(fabsf(ch[k]), fabsf(xh[k]), b);
        const float sg = sigma_of(b);
        /* the bounded sum (dfs_mul, then dfs_fma) */
        float tau = 0.0f, lo = 0.0f;
        double tau_exact = 0.0; /* the q's summed in double: exact (all multiples of 2^-24 sigma) */
        for (int k = 0; k < n; ++k) {
            const float p = ch[k] * xh[k];
            const float q = (sg + p) - sg;
            const float r = fmaf(ch[k], xh[k], -q);
            tau_exact += (double)q;
            if (k == 0) {
                tau = q;
                lo = fmaf(cl[k], xh[k], fmaf(ch[k], xl[k], r));
            } else {
                tau = tau + q;
                lo = fmaf(cl[k], xh[k], fmaf(ch[k], xl[k], lo + r));
            }
            if ((double)tau != tau_exact) {
                if (bad < 5) fprintf(stderr, "trial %ld term %d: partial sum of q not exact\n", t, k);
                ++bad;
            }
        }
        /* renorm: TwoSum(tau, lo) */
        const float s = tau + lo, v = s - tau;
        const float e = (tau - (s - v)) + (lo - v);
        /* exact value of sum (ch + cl)(xh + xl) */
        quad ex = 0;
        for (int k = 0; k < n; ++k)
            ex += ((quad)ch[k] + (quad)cl[k]) * ((quad)xh[k] + (quad)xl[k]);
        const quad got = (quad)s + (quad)e;
        quad err = got - ex;
        if (err < 0) err = -err;
        const double rel = b > 0 ? (double)(err / (quad)b) : 0.0;
        const double bound = (double)n * n * ldexp(1.0, -46);
        if (rel > worst[si]) worst[si] = rel;
        if (rel > bound) {
            if (bad < 5) fprintf(stderr, "trial %ld (n=%d): error %.3e B above the bound %.3e B\n", t, n, rel, bound);
            ++bad;
        }
    }
    for (int i = 0; i < 6; ++i) printf("n=%d worst_error_over_B=%.3e bound=%.3e\n", sizes[i], worst[i],
                                       (double)sizes[i] * sizes[i] * ldexp(1.0, -46));
    printf("violations=%ld\n", bad);
    return bad ? 1 : 0;
}
