/*
 * ORACLE -- test infrastructure only.  Nothing in the product links this file;
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.
 *
 * Double-precision reference for the transform the reference computes
 * (larsjoost/wgls-rs-fft src/lib.rs:433-488): forward X_k = sum_n x_n
 * e^{-2 pi i k n / N}, unscaled; inverse with e^{+2 pi i k n / N} and 1/N
 * (src/lib.rs:571-579 + 661-669 give conj(DFT(conj x))/N, which is that).
 *
 * Twiddles are produced from the exact rational j/N: the angle is reduced to
 * the first octant by integer arithmetic before sin/cos are evaluated, so
 * every twiddle is within one ulp of double.  The FFT is a radix-2 Stockham
 * autosort in double (O(N log N)); fft64_dft is the O(N^2) direct sum that
 * pins it for N <= 4096.
 */
#define _GNU_SOURCE /* pthread_barrier_t under -std=c11 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

static const double PI_D = 3.14159265358979323846264338327950288;

/* e^{-2 pi i j / n} for integer j, with exact octant reduction. */
void fft64_twiddle(uint64_t j, uint64_t n, double *c, double *s)
{
    j %= n;
    /* angle = 2 pi j / n = (pi/4) * (8 j / n); split 8j = q*n + r. */
    unsigned __int128 j8 = (unsigned __int128)j * 8u;
    uint64_t q = (uint64_t)(j8 / n);
    uint64_t r = (uint64_t)(j8 % n);
    /* theta in [0, pi/4): theta = (pi/4) * r / n */
    double frac = (double)r / (double)n; /* exact for n a power of two */
    int odd = (int)(q & 1u);
    double t = odd ? (1.0 - frac) : frac;
    double th = (PI_D / 4.0) * t;
    double sn = sin(th), cs = cos(th);
    /* (cos, sin) of the full angle from the octant index q. */
    double C, S;
    switch (q & 7u) {
    case 0: C = cs;  S = sn;  break;
    case 1: C = sn;  S = cs;  break;
    case 2: C = -sn; S = cs;  break;
    case 3: C = -cs; S = sn;  break;
    case 4: C = -cs; S = -sn; break;
    case 5: C = -sn; S = -cs; break;
    case 6: C = sn;  S = -cs; break;
    default: C = cs; S = -sn; break;
    }
    *c = C;
    *s = -S; /* forward kernel: e^{-i angle} */
}

/* In/out: interleaved double complex, one transform of length n. */
static void stockham64(double *x, double *y, const double *tw, uint64_t n, int inverse)
{
    /* radix-2 Stockham: stage with p = 1,2,4,...,n/2 */
    double *src = x, *dst = y;
    uint64_t half = n >> 1;
    for (uint64_t p = 1; p < n; p <<= 1) {
        for (uint64_t tid = 0; tid < half; ++tid) {
            uint64_t k = tid & (p - 1), j = tid / p;
            uint64_t i1 = j * p + k, i2 = i1 + half;
            double ar = src[2 * i1], ai = src[2 * i1 + 1];
            double br = src[2 * i2], bi = src[2 * i2 + 1];
            uint64_t t = k * (half / p);
            double wr = tw[2 * t], wi = tw[2 * t + 1];
            if (inverse)
                wi = -wi;
            double tr = wr * br - wi * bi, ti = wr * bi + wi * br;
            uint64_t d = 2 * (j * 2 * p + k);
            dst[d] = ar + tr;
            dst[d + 1] = ai + ti;
            dst[d + 2 * p] = ar - tr;
            dst[d + 2 * p + 1] = ai - ti;
        }
        double *tmp = src; src = dst; dst = tmp;
    }
    if (src != x)
        memcpy(x, src, n * 2 * sizeof(double));
}

typedef struct {
    const float *in_f;
    const double *in_d;
    double *out;
    const double *tw;
    uint64_t n, row0, rows;
    int inverse;
} f64_job;

static void *f64_worker(void *arg)
{
    f64_job *j = (f64_job *)arg;
    uint64_t n = j->n;
    double *x = (double *)malloc(n * 2 * sizeof(double));
    double *y = (double *)malloc(n * 2 * sizeof(double));
    if (!x || !y) {
        free(x); free(y);
        return (void *)1;
    }
    for (uint64_t r = j->row0; r < j->row0 + j->rows; ++r) {
        for (uint64_t i = 0; i < 2 * n; ++i)
            x[i] = j->in_f ? (double)j->in_f[r * 2 * n + i] : j->in_d[r * 2 * n + i];
        if (n > 1)
            stockham64(x, y, j->tw, n, j->inverse);
        double sc = j->inverse ? 1.0 / (double)n : 1.0;
        for (uint64_t i = 0; i < 2 * n; ++i)
            j->out[r * 2 * n + i] = x[i] * sc;
    }
    free(x); free(y);
    return NULL;
}

/* One long transform split over threads stage by stage (batches smaller than
 * the thread count, e.g. a single 2^26-point row): each thread takes a
 * contiguous range of butterflies of every radix-2 stage, with a barrier
 * between stages.  Same arithmetic as stockham64, so the same result. */
typedef struct {
    const float *in_f;
    const double *in_d;
    double *out, *x, *y, *tw;
    uint64_t n, row;
    int inverse, t, threads;
    pthread_barrier_t *bar;
} f64_stage_job;

static void *f64_stage_worker(void *arg)
{
    f64_stage_job *j = (f64_stage_job *)arg;
    uint64_t n = j->n, half = n >> 1;
    uint64_t lo = half * (uint64_t)j->t / (uint64_t)j->threads;
    uint64_t hi = half * (uint64_t)(j->t + 1) / (uint64_t)j->threads;
    for (uint64_t i = 2 * lo; i < 2 * hi; ++i) { /* load this thread's share of the row */
        uint64_t a = i, b = i + n;
        j->x[a] = j->in_f ? (double)j->in_f[j->row * 2 * n + a] : j->in_d[j->row * 2 * n + a];
        j->x[b] = j->in_f ? (double)j->in_f[j->row * 2 * n + b] : j->in_d[j->row * 2 * n + b];
    }
    pthread_barrier_wait(j->bar);
    double *src = j->x, *dst = j->y;
    for (uint64_t p = 1; p < n; p <<= 1) {
        for (uint64_t tid = lo; tid < hi; ++tid) {
            uint64_t k = tid & (p - 1), jj = tid / p;
            uint64_t i1 = jj * p + k, i2 = i1 + half;
            double ar = src[2 * i1], ai = src[2 * i1 + 1];
            double br = src[2 * i2], bi = src[2 * i2 + 1];
            uint64_t t = k * (half / p);
            double wr = j->tw[2 * t], wi = j->tw[2 * t + 1];
            if (j->inverse)
                wi = -wi;
            double tr = wr * br - wi * bi, ti = wr * bi + wi * br;
            uint64_t d = 2 * (jj * 2 * p + k);
            dst[d] = ar + tr;
            dst[d + 1] = ai + ti;
            dst[d + 2 * p] = ar - tr;
            dst[d + 2 * p + 1] = ai - ti;
        }
        pthread_barrier_wait(j->bar);
        double *tmp = src; src = dst; dst = tmp;
    }
    double sc = j->inverse ? 1.0 / (double)n : 1.0;
    for (uint64_t i = 2 * lo; i < 2 * hi; ++i) {
        j->out[j->row * 2 * n + i] = src[i] * sc;
        j->out[j->row * 2 * n + i + n] = src[i + n] * sc;
    }
    return NULL;
}

static int fft64_rows_stage_parallel(const float *in_f, const double *in_d, double *out, double *tw,
                                     uint64_t n, uint64_t batch, int inverse, int threads)
{
    double *x = (double *)malloc(n * 2 * sizeof(double));
    double *y = (double *)malloc(n * 2 * sizeof(double));
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * threads);
    f64_stage_job *jobs = (f64_stage_job *)malloc(sizeof(f64_stage_job) * threads);
    int rc = 0;
    if (!x || !y || !th || !jobs) {
        rc = -2;
    } else {
        pthread_barrier_t bar;
        for (uint64_t r = 0; r < batch; ++r) {
            pthread_barrier_init(&bar, NULL, (unsigned)threads);
            for (int t = 0; t < threads; ++t) {
                jobs[t] = (f64_stage_job){in_f, in_d, out, x, y, tw, n, r, inverse, t, threads, &bar};
                pthread_create(&th[t], NULL, f64_stage_worker, &jobs[t]);
            }
            for (int t = 0; t < threads; ++t)
                pthread_join(th[t], NULL);
            pthread_barrier_destroy(&bar);
        }
    }
    free(x); free(y); free(th); free(jobs);
    return rc;
}

static int fft64_batch_impl(const float *in_f, const double *in_d, double *out,
                            uint64_t n, uint64_t batch, int inverse, int threads)
{
    if (n == 0 || (n & (n - 1)) != 0)
        return -1;
    double *tw = (double *)malloc((n / 2 + 1) * 2 * sizeof(double));
    if (!tw)
        return -2;
    for (uint64_t j = 0; j < n / 2 + 1; ++j)
        fft64_twiddle(j, n, &tw[2 * j], &tw[2 * j + 1]);
    if (threads < 1)
        threads = 1;
    if ((uint64_t)threads > 2 * batch && n >= (1u << 16) && (uint64_t)threads <= n / 2) {
        int rc = fft64_rows_stage_parallel(in_f, in_d, out, tw, n, batch, inverse, threads);
        free(tw);
        return rc;
    }
    if ((uint64_t)threads > batch)
        threads = (int)(batch ? batch : 1);
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * threads);
    f64_job *jobs = (f64_job *)malloc(sizeof(f64_job) * threads);
    uint64_t done = 0;
    int rc = 0;
    for (int t = 0; t < threads; ++t) {
        uint64_t rows = batch / threads + ((uint64_t)t < batch % threads ? 1 : 0);
        jobs[t] = (f64_job){in_f, in_d, out, tw, n, done, rows, inverse};
        pthread_create(&th[t], NULL, f64_worker, &jobs[t]);
        done += rows;
    }
    for (int t = 0; t < threads; ++t) {
        void *ret = NULL;
        pthread_join(th[t], &ret);
        if (ret)
            rc = -2;
    }
    free(th); free(jobs); free(tw);
    return rc;
}

/* float32 interleaved input -> double interleaved output. */
int fft64_batch_f32in(const float *in, double *out, uint64_t n, uint64_t batch,
                      int inverse, int threads)
{
    return fft64_batch_impl(in, NULL, out, n, batch, inverse, threads);
}

/* double interleaved input -> double interleaved output. */
int fft64_batch(const double *in, double *out, uint64_t n, uint64_t batch,
                int inverse, int threads)
{
    return fft64_batch_impl(NULL, in, out, n, batch, inverse, threads);
}

/* Direct O(N^2) DFT in double with the same exact twiddles (one row). */
int fft64_dft(const double *in, double *out, uint64_t n, int inverse)
{
    if (n == 0)
        return -1;
    double *tw = (double *)malloc(n * 2 * sizeof(double));
    if (!tw)
        return -2;
    for (uint64_t j = 0; j < n; ++j)
        fft64_twiddle(j, n, &tw[2 * j], &tw[2 * j + 1]);
    for (uint64_t k = 0; k < n; ++k) {
        double sr = 0.0, si = 0.0;
        for (uint64_t m = 0; m < n; ++m) {
            uint64_t e = (k * m) % n;
            double wr = tw[2 * e], wi = inverse ? -tw[2 * e + 1] : tw[2 * e + 1];
            double xr = in[2 * m], xi = in[2 * m + 1];
            sr += xr * wr - xi * wi;
            si += xr * wi + xi * wr;
        }
        double sc = inverse ? 1.0 / (double)n : 1.0;
        out[2 * k] = sr * sc;
        out[2 * k + 1] = si * sc;
    }
    free(tw);
    return 0;
}
