/*
 * ORACLE -- test infrastructure only.  Nothing in the product links this file;
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.
 *
 * CPU restatement of the reference's own FFT path (larsjoost/wgls-rs-fft,
 * the "Baseline (Stockham Radix-4/2)" executor) in single precision:
 *
 *   twiddle table     src/lib.rs:761-769   f32 cos/sin of the f32 angle
 *                                          (-TAU * j) / n, j < n
 *   stage schedule    src/lib.rs:724-731   floor(log4 N) radix-4 stages with
 *                     src/lib.rs:836-861   p = 4^s, one radix-2 stage with
 *                                          p = 4^floor(log4 N) if log2 N is odd
 *   ping-pong         src/lib.rs:863-899   stage s reads A (s even) or B, result
 *                                          lands in B when the stage count is odd
 *   radix-4 stage     src/shaders.rs:8-63
 *   radix-2 stage     src/shaders.rs:69-106
 *   input prep        src/lib.rs:571-579   interleave, conjugate for the inverse
 *   inverse post      src/lib.rs:661-669   conjugate and multiply by 1.0f/n
 *   batch driver      src/lib.rs:517-568
 *
 * Known reference defect NOT reproduced: for N == 2 the reference computes
 * zero radix-4 workgroups, takes its legacy dispatch branch and skips the
 * radix-2 stage while still reading buffer B (src/lib.rs:595-614, 899-902), so
 * it returns an unwritten buffer.  This restatement runs the radix-2 stage and
 * returns the correct 2-point DFT.  N == 1 is the identity in both.
 *
 * Build with -ffp-contract=off so every multiply and add rounds separately,
 * as the WGSL source spells them.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define REF_TAU_F 6.28318530717958647692f /* std::f32::consts::TAU */

/* src/lib.rs:764-769: angle = -TAU * j as f32 / n as f32; [cos, sin]. */
void ref_twiddles(uint32_t n, float *tw /* 2*n floats */)
{
    for (uint32_t j = 0; j < n; ++j) {
        float angle = (-REF_TAU_F * (float)j) / (float)n;
        tw[2 * j] = cosf(angle);
        tw[2 * j + 1] = sinf(angle);
    }
}

static inline void cmul(float ar, float ai, float br, float bi, float *cr, float *ci)
{
    /* src/shaders.rs:16-18: vec2(a.x*b.x - a.y*b.y, a.x*b.y + a.y*b.x) */
    float t0 = ar * br;
    float t1 = ai * bi;
    float t2 = ar * bi;
    float t3 = ai * br;
    *cr = t0 - t1;
    *ci = t2 + t3;
}

/* One radix-4 Stockham stage over `batch` transforms (src/shaders.rs:20-62). */
void ref_r4_stage(const float *src, float *dst, const float *tw, uint32_t n,
                  uint32_t p, uint32_t batch)
{
    const uint32_t quarter_n = n >> 2;
    const uint32_t four_p = p << 2;
    for (uint32_t b = 0; b < batch; ++b) {
        const float *s = src + (size_t)b * n * 2;
        float *d = dst + (size_t)b * n * 2;
        for (uint32_t tid = 0; tid < quarter_n; ++tid) {
            uint32_t k = tid % p, j = tid / p;
            uint32_t i0 = j * p + k, i1 = i0 + quarter_n, i2 = i1 + quarter_n,
                     i3 = i2 + quarter_n;
            float x0r = s[2 * i0], x0i = s[2 * i0 + 1];
            float x1r = s[2 * i1], x1i = s[2 * i1 + 1];
            float x2r = s[2 * i2], x2i = s[2 * i2 + 1];
            float x3r = s[2 * i3], x3i = s[2 * i3 + 1];
            uint32_t stride = quarter_n / p, t = k * stride;
            cmul(tw[2 * t], tw[2 * t + 1], x1r, x1i, &x1r, &x1i);
            cmul(tw[4 * t], tw[4 * t + 1], x2r, x2i, &x2r, &x2i);
            cmul(tw[6 * t], tw[6 * t + 1], x3r, x3i, &x3r, &x3i);
            float s02r = x0r + x2r, s02i = x0i + x2i;
            float d02r = x0r - x2r, d02i = x0i - x2i;
            float s13r = x1r + x3r, s13i = x1i + x3i;
            float d13r = x1r - x3r, d13i = x1i - x3i;
            uint32_t db = 2 * (j * four_p + k);
            d[db] = s02r + s13r;
            d[db + 1] = s02i + s13i;
            d[db + 2 * p] = d02r + d13i;
            d[db + 2 * p + 1] = d02i - d13r;
            d[db + 4 * p] = s02r - s13r;
            d[db + 4 * p + 1] = s02i - s13i;
            d[db + 6 * p] = d02r - d13i;
            d[db + 6 * p + 1] = d02i + d13r;
        }
    }
}

/* Final radix-2 Stockham stage when log2 N is odd (src/shaders.rs:81-105). */
void ref_r2_stage(const float *src, float *dst, const float *tw, uint32_t n,
                  uint32_t p, uint32_t batch)
{
    const uint32_t half_n = n >> 1;
    const uint32_t two_p = p + p;
    for (uint32_t b = 0; b < batch; ++b) {
        const float *s = src + (size_t)b * n * 2;
        float *d = dst + (size_t)b * n * 2;
        for (uint32_t tid = 0; tid < half_n; ++tid) {
            uint32_t k = tid % p, j = tid / p;
            uint32_t i1 = j * p + k, i2 = i1 + half_n;
            float x1r = s[2 * i1], x1i = s[2 * i1 + 1];
            float x2r = s[2 * i2], x2i = s[2 * i2 + 1];
            uint32_t t = k * (half_n / p);
            float tr, ti;
            cmul(tw[2 * t], tw[2 * t + 1], x2r, x2i, &tr, &ti);
            uint32_t db = 2 * (j * two_p + k);
            d[db] = x1r + tr;
            d[db + 1] = x1i + ti;
            d[db + 2 * p] = x1r - tr;
            d[db + 2 * p + 1] = x1i - ti;
        }
    }
}

/*
 * The reference's forward pass over an interleaved batch held in buf_a
 * (src/lib.rs:582-628 with the schedule of src/lib.rs:724-731,836-899).
 * Returns a pointer to the buffer holding the result (buf_a or buf_b).
 */
float *ref_execute(float *buf_a, float *buf_b, const float *tw, uint32_t n,
                   uint32_t batch)
{
    if (n <= 1)
        return buf_a;
    uint32_t log_n = 0;
    while ((1u << log_n) < n)
        ++log_n;
    uint32_t num_r4 = log_n / 2;
    int has_r2 = (log_n % 2) == 1;
    float *src = buf_a, *dst = buf_b;
    for (uint32_t s = 0; s < num_r4; ++s) {
        ref_r4_stage(src, dst, tw, n, 1u << (2 * s), batch);
        float *t = src; src = dst; dst = t;
    }
    if (has_r2) {
        ref_r2_stage(src, dst, tw, n, 1u << (2 * num_r4), batch);
        float *t = src; src = dst; dst = t;
    }
    return src;
}

/* src/lib.rs:571-579 */
void ref_prepare_input(const float *in, uint64_t count, int inverse, float *out)
{
    for (uint64_t i = 0; i < count; ++i) {
        out[2 * i] = in[2 * i];
        out[2 * i + 1] = inverse ? -in[2 * i + 1] : in[2 * i + 1];
    }
}

/* src/lib.rs:661-669 */
void ref_inverse_post(float *data, uint64_t count, uint32_t n)
{
    float scale = 1.0f / (float)n;
    for (uint64_t i = 0; i < count; ++i) {
        data[2 * i] = data[2 * i] * scale;
        data[2 * i + 1] = -data[2 * i + 1] * scale;
    }
}

/* Full transform_batch_internal (src/lib.rs:517-568) over an interleaved
 * batch: in/out are batch*n complex values.  Returns 0, or -1 on bad size. */
int ref_fft_batch(const float *in, float *out, uint32_t n, uint32_t batch, int inverse)
{
    if (n == 0 || (n & (n - 1)) != 0)
        return -1;
    size_t cnt = (size_t)n * batch;
    float *a = (float *)malloc(cnt * 2 * sizeof(float));
    float *b = (float *)malloc(cnt * 2 * sizeof(float));
    float *tw = (float *)malloc((size_t)n * 2 * sizeof(float));
    if (!a || !b || !tw) {
        free(a); free(b); free(tw);
        return -2;
    }
    ref_twiddles(n, tw);
    ref_prepare_input(in, cnt, inverse, a);
    float *res = ref_execute(a, b, tw, n, batch);
    if (inverse)
        ref_inverse_post(res, cnt, n);
    memcpy(out, res, cnt * 2 * sizeof(float));
    free(a); free(b); free(tw);
    return 0;
}

/* ---- threaded driver (CPU baseline timing): rows split across threads ---- */
typedef struct {
    const float *in;
    float *out;
    const float *tw;
    uint32_t n, rows;
    int inverse;
    float *scratch; /* 4*n*rows floats */
} ref_job;

static void *ref_worker(void *arg)
{
    ref_job *j = (ref_job *)arg;
    size_t cnt = (size_t)j->n * j->rows;
    float *a = j->scratch, *b = j->scratch + cnt * 2;
    ref_prepare_input(j->in, cnt, j->inverse, a);
    float *res = ref_execute(a, b, j->tw, j->n, j->rows);
    if (j->inverse)
        ref_inverse_post(res, cnt, j->n);
    memcpy(j->out, res, cnt * 2 * sizeof(float));
    return NULL;
}

/* Same result as ref_fft_batch; the batch is split into `threads` slices. */
int ref_fft_batch_mt(const float *in, float *out, uint32_t n, uint32_t batch,
                     int inverse, int threads)
{
    if (n == 0 || (n & (n - 1)) != 0)
        return -1;
    if (threads < 1)
        threads = 1;
    if ((uint32_t)threads > batch)
        threads = (int)batch;
    if (threads <= 1)
        return ref_fft_batch(in, out, n, batch, inverse);
    float *tw = (float *)malloc((size_t)n * 2 * sizeof(float));
    float *scratch = (float *)malloc((size_t)n * batch * 4 * sizeof(float));
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * threads);
    ref_job *jobs = (ref_job *)malloc(sizeof(ref_job) * threads);
    if (!tw || !scratch || !th || !jobs) {
        free(tw); free(scratch); free(th); free(jobs);
        return -2;
    }
    ref_twiddles(n, tw);
    uint32_t done = 0;
    for (int t = 0; t < threads; ++t) {
        uint32_t rows = batch / threads + ((uint32_t)t < batch % threads ? 1 : 0);
        size_t off = (size_t)done * n;
        jobs[t].in = in + off * 2;
        jobs[t].out = out + off * 2;
        jobs[t].tw = tw;
        jobs[t].n = n;
        jobs[t].rows = rows;
        jobs[t].inverse = inverse;
        jobs[t].scratch = scratch + off * 4;
        pthread_create(&th[t], NULL, ref_worker, &jobs[t]);
        done += rows;
    }
    for (int t = 0; t < threads; ++t)
        pthread_join(th[t], NULL);
    free(tw); free(scratch); free(th); free(jobs);
    return 0;
}
