/*
 * uhs_oracle.c -- CPU restatement of UHStencil's serial stencil loops.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker that the CUDA sweep
 * kernels are compared against.  It is loaded by the tests, by
 * __graft_entry__.smoke() and by the cpu_baseline leg of bench.py, and by
 * nothing else; the library under uxxxxxxxxh_gb300/ never links or calls it.
 *
 * What it restates (reference paths are inside the UHStencil project):
 *   - mpe_verify() in UH-SW/<case>/stencil_<n>pt_driver.serial.c, e.g.
 *     UH-SW/3d1r_star/stencil_3d7pt_driver.serial.c:38-89 and
 *     UH-SW/2d1r_star/stencil_2d5pt_driver.serial.c:36-80, and its twin
 *     cpu_verify() in UH-GPU/<case>/<n>pt_main.cpp:50-103:
 *       for iter < T/2 { sweep(in -> tmp); sweep(tmp -> in) }
 *     where one sweep visits every point of the domain [lb, ub) (slowest axis
 *     first) and stores  sum_k c_k * in[p + o_k]  evaluated left to right in
 *     the order the terms are written in the stencil's .dsl expression.
 *     Points outside the domain (the halo) are never written.
 *   - A single sweep (T == 1) is the compute function MLIRGen emits without
 *     an iteration wrapper (UHStencil/lib/Parser/MLIRGen.cpp:317-352): one
 *     sweep in -> out.
 *   - The rand() % 50 initialisation of every cell of all four arrays done by
 *     the drivers' main() (e.g. UH-SW/3d1r_star/stencil_3d7pt_driver.serial.c:96-105).
 *
 * Build: gcc -O2 -ffp-contract=off -fopenmp (see oracle/Makefile).  No FMA
 * contraction, so every product and every sum is rounded separately, exactly
 * as the reference drivers compiled with the same flags.  OpenMP splits the
 * two outer loops across threads; every point is written by one thread from
 * values of the previous sweep only, so results are bit-identical for any
 * thread count.
 *
 * Parity pin: tests/test_oracle_pin.py checks this restatement bit-for-bit
 * against the unmodified reference drivers compiled by oracle/Makefile into
 * oracle/_ref/, and tests/golden/ holds the digests that pin made.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* One stencil program in the oracle's terms.  Rank-2 grids use sizes[0]=1,
 * lb[0]=0, ub[0]=1 and dz=0 for every term. */
typedef struct {
    int64_t sizes[3];   /* padded extents, slowest axis first */
    int64_t lb[3];      /* domain lower bounds (inclusive) */
    int64_t ub[3];      /* domain upper bounds (exclusive) */
    int32_t nterms;
    const int32_t *off; /* nterms x (dz, dy, dx) in expression order */
    const double *coef; /* nterms coefficients in expression order */
} oracle_stencil;

void oracle_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int oracle_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* One sweep, FP64: out[p] = ((c0*in[p+o0] + c1*in[p+o1]) + c2*in[p+o2]) + ... */
void oracle_sweep_f64(const oracle_stencil *s, const double *in, double *out)
{
    const int64_t sy = s->sizes[2], sz = s->sizes[1] * s->sizes[2];
    const int nt = s->nterms;
    int64_t *delta = (int64_t *)malloc(sizeof(int64_t) * (size_t)(nt > 0 ? nt : 1));
    for (int t = 0; t < nt; t++)
        delta[t] = s->off[3 * t] * sz + s->off[3 * t + 1] * sy + s->off[3 * t + 2];
    const int64_t z0 = s->lb[0], z1 = s->ub[0], y0 = s->lb[1], y1 = s->ub[1];
    const int64_t x0 = s->lb[2], x1 = s->ub[2];
#pragma omp parallel for collapse(2) schedule(static)
    for (int64_t z = z0; z < z1; z++) {
        for (int64_t y = y0; y < y1; y++) {
            const int64_t row = z * sz + y * sy;
            for (int64_t x = x0; x < x1; x++) {
                const double *p = in + row + x;
                double acc = s->coef[0] * p[delta[0]];
                for (int t = 1; t < nt; t++)
                    acc = acc + s->coef[t] * p[delta[t]];
                out[row + x] = acc;
            }
        }
    }
    free(delta);
}

/* The generated <name>_iteration entry: T == 1 is one sweep a -> b; an even T
 * runs T/2 pairs (a -> b, b -> a) and leaves step T in a and step T-1 in b.
 * Odd T > 1 is rejected, as MLIRGen does (MLIRGen.cpp:317-321). */
int oracle_iterate_f64(const oracle_stencil *s, double *a, double *b, int T)
{
    if (T == 1) {
        oracle_sweep_f64(s, a, b);
        return 0;
    }
    if (T < 0 || (T % 2) != 0) return -1;
    for (int it = 0; it < T / 2; it++) {
        oracle_sweep_f64(s, a, b);
        oracle_sweep_f64(s, b, a);
    }
    return 0;
}

/* Plain single sweeps in FP32 arithmetic (products and sums rounded to
 * float).  Used only to bound what an FP32 kernel can be expected to reach. */
void oracle_sweep_f32(const oracle_stencil *s, const float *in, float *out)
{
    const int64_t sy = s->sizes[2], sz = s->sizes[1] * s->sizes[2];
    const int nt = s->nterms;
    int64_t *delta = (int64_t *)malloc(sizeof(int64_t) * (size_t)(nt > 0 ? nt : 1));
    float *cf = (float *)malloc(sizeof(float) * (size_t)(nt > 0 ? nt : 1));
    for (int t = 0; t < nt; t++) {
        delta[t] = s->off[3 * t] * sz + s->off[3 * t + 1] * sy + s->off[3 * t + 2];
        cf[t] = (float)s->coef[t];
    }
#pragma omp parallel for collapse(2) schedule(static)
    for (int64_t z = s->lb[0]; z < s->ub[0]; z++) {
        for (int64_t y = s->lb[1]; y < s->ub[1]; y++) {
            const int64_t row = z * sz + y * sy;
            for (int64_t x = s->lb[2]; x < s->ub[2]; x++) {
                const float *p = in + row + x;
                float acc = cf[0] * p[delta[0]];
                for (int t = 1; t < nt; t++)
                    acc = acc + cf[t] * p[delta[t]];
                out[row + x] = acc;
            }
        }
    }
    free(delta);
    free(cf);
}

/* The drivers' main(): every cell of every array gets rand() % 50, cell by
 * cell, writing the same value into all arrays before drawing the next one.
 * The drivers never seed, which is the state srand(1) restores. */
void oracle_fill_rand50(double **arrays, int narrays, int64_t n)
{
    srand(1);
    for (int64_t i = 0; i < n; i++) {
        double v = rand() % 50;
        for (int a = 0; a < narrays; a++) arrays[a][i] = v;
    }
}

/* Error of x against the oracle r over the domain of s:
 *   out[0] = ||x - r||_2 / ||r||_2     (relative L2)
 *   out[1] = max |x - r|               (max absolute)
 *   out[2] = max |x - r| / max |r|     (max error relative to the field's scale)
 *   out[3] = max |r|
 * Accumulated in long double so the metric itself adds no error at the
 * 1e-15 level. */
void oracle_error_f64(const oracle_stencil *s, const double *r, const double *x, double *out)
{
    const int64_t sy = s->sizes[2], sz = s->sizes[1] * s->sizes[2];
    long double num = 0.0L, den = 0.0L;
    double maxabs = 0.0, maxref = 0.0;
    for (int64_t z = s->lb[0]; z < s->ub[0]; z++)
        for (int64_t y = s->lb[1]; y < s->ub[1]; y++)
            for (int64_t xx = s->lb[2]; xx < s->ub[2]; xx++) {
                const int64_t i = z * sz + y * sy + xx;
                const double d = x[i] - r[i];
                num += (long double)d * d;
                den += (long double)r[i] * r[i];
                if (fabs(d) > maxabs || d != d) maxabs = (d != d) ? INFINITY : fabs(d);
                if (fabs(r[i]) > maxref) maxref = fabs(r[i]);
            }
    out[0] = den > 0 ? (double)sqrtl(num / den) : (double)sqrtl(num);
    out[1] = maxabs;
    out[2] = maxref > 0 ? maxabs / maxref : maxabs;
    out[3] = maxref;
}

/* Same metric for an FP32 result against the FP64 oracle. */
void oracle_error_f32(const oracle_stencil *s, const double *r, const float *x, double *out)
{
    const int64_t sy = s->sizes[2], sz = s->sizes[1] * s->sizes[2];
    long double num = 0.0L, den = 0.0L;
    double maxabs = 0.0, maxref = 0.0;
    for (int64_t z = s->lb[0]; z < s->ub[0]; z++)
        for (int64_t y = s->lb[1]; y < s->ub[1]; y++)
            for (int64_t xx = s->lb[2]; xx < s->ub[2]; xx++) {
                const int64_t i = z * sz + y * sy + xx;
                const double d = (double)x[i] - r[i];
                num += (long double)d * d;
                den += (long double)r[i] * r[i];
                if (fabs(d) > maxabs || d != d) maxabs = (d != d) ? INFINITY : fabs(d);
                if (fabs(r[i]) > maxref) maxref = fabs(r[i]);
            }
    out[0] = den > 0 ? (double)sqrtl(num / den) : (double)sqrtl(num);
    out[1] = maxabs;
    out[2] = maxref > 0 ? maxabs / maxref : maxabs;
    out[3] = maxref;
}

/* Number of cells outside the domain whose bytes differ between a and b
 * (the halo must come back bit-exact). */
int64_t oracle_halo_diff_bytes(const oracle_stencil *s, const void *a, const void *b, int64_t elem)
{
    const int64_t sy = s->sizes[2], sz = s->sizes[1] * s->sizes[2];
    int64_t bad = 0;
    const unsigned char *pa = (const unsigned char *)a, *pb = (const unsigned char *)b;
    for (int64_t z = 0; z < s->sizes[0]; z++)
        for (int64_t y = 0; y < s->sizes[1]; y++)
            for (int64_t x = 0; x < s->sizes[2]; x++) {
                const int inside = z >= s->lb[0] && z < s->ub[0] && y >= s->lb[1] && y < s->ub[1] &&
                                   x >= s->lb[2] && x < s->ub[2];
                if (inside) continue;
                const int64_t i = (z * sz + y * sy + x) * elem;
                if (memcmp(pa + i, pb + i, (size_t)elem) != 0) bad++;
            }
    return bad;
}
