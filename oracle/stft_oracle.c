/*
 * TEST INFRASTRUCTURE ONLY — CPU oracle for OCCAstft's STFT hot path.
 *
 * Used by tests/, __graft_entry__.smoke() and bench.py's CPU legs as the
 * checker / the timed CPU baseline.  The product never links it.
 *
 * Parity status: PINNED.  orc_serial_pipeline is checked bit-for-bit against
 * the reference's own Serial and OpenMP runner code compiled from source by
 * oracle/build_ref.sh (tests/test_oracle_ref.py) and against the committed
 * golden vectors in tests/golden/ (tests/test_oracle_golden.py).
 *
 * Every float/double conversion below mirrors the reference's translated
 * serial kernels; build with -ffp-contract=off so that no multiply-add is
 * fused (the reference's x86 build issues none).
 *
 * Reference files cited (paths inside the OCCAstft project):
 *   StandAlone/cross_gpgpu/GLOBAL/RunnerInterface.hpp:26-35     toQuot
 *   StandAlone/cross_gpgpu/Serial/src/SerialImpl.cpp:36-51      sizes, buffers
 *   StandAlone/cross_gpgpu/GLOBAL/RunnerCommon.cpp:166-318      Default_Pipeline
 *   StandAlone/cross_gpgpu/Serial/src/functionImpl.cpp:207-303  EXPC, ToPower
 *   OKL/kernel.okl:33-127        window formulas
 *   OKL/kernel.okl:141-218       segmentK, twiddle, toPower, toHalfComplexFormat
 *   OKL/EXPCommon.okl:7-27       Overlap_Common
 *   OKL/EXPCommon.okl:151-192    DCRemove_Common
 *   OKL/EXPCommon.okl:194-245    StockHamCommon (radix-2 Stockham stage)
 */
#include "stft_oracle.h"

#include <errno.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_PI 3.14159265358979323846

/* ------------------------------------------------------------------ */
/* geometry: RunnerInterface.hpp:26-35 (float arithmetic, truncation)  */
/* ------------------------------------------------------------------ */
static int orc_to_quot(float full, float ov, float win)
{
    if (ov == 0.0f) {
        float q = full / win + 1.0f;
        return (int)q;
    }
    float q = full / (win * (1.0f - ov)) + 1.0f;
    return (int)q;
}

int orc_geometry_get(uint32_t n, int exp, float overlap, orc_geometry* g)
{
    if (exp < 6 || exp > 30) return -1;
    if (!(overlap < 1.0f)) return -1;               /* OMove would be 0: toQuot divides by 0 */
    const int win = 1 << exp;
    /* SerialImpl.cpp:42  OMove = windowSize * (1.0f - overlapRatio) */
    const float hopf = (float)win * (1.0f - overlap);
    if (!(hopf >= 1.0f) || hopf >= 4294967296.0f) return -1;
    const uint32_t hop = (uint32_t)hopf;
    const float qf = (float)n / ((float)win * (1.0f - overlap)) + 1.0f;
    if (!(qf < 2147483648.0f)) return -1;
    const int qt = orc_to_quot((float)n, overlap, (float)win);
    const uint64_t ofull = (uint64_t)(uint32_t)qt * (uint64_t)win;
    if (qt <= 0 || ofull >= 4294967296ull) return -1;
    g->qt = (uint32_t)qt;
    g->hop = hop;
    g->ofull = (uint32_t)ofull;
    g->ohalf = (uint32_t)(ofull / 2);
    g->n_window = (uint32_t)win;
    return 0;
}

/* ------------------------------------------------------------------ */
/* options: RunnerCommon.cpp:216-253                                   */
/* ------------------------------------------------------------------ */
static void orc_set_err(char* err, size_t cap, const char* msg)
{
    if (err && cap) {
        strncpy(err, msg, cap - 1);
        err[cap - 1] = 0;
    }
}

int orc_parse_options(const char* options, orc_options* o, char* err, size_t errcap)
{
    memset(o, 0, sizeof(*o));
    o->sigma = -1.0f;
    if (!options) options = "";
    static const char* kWin[] = {
        "--hanning_window", "--hamming_window", "--blackman_window",
        "--nuttall_window", "--blackman_nuttall_window",
        "--blackman_harris_window", "--flattop_window"};
    for (int i = 0; i < 7; ++i) {
        if (strstr(options, kWin[i])) { o->window = i + 1; break; }
    }
    if (o->window == ORC_WIN_NONE) {
        const char* gpos = strstr(options, "--gaussian_window=");
        const char* spos = strstr(options, "<<sigma");
        if (gpos && spos) {
            /* the reference starts the sigma text 19 characters after an
             * 18-character prefix, skipping the first sigma character */
            const size_t len = strlen(options);
            const size_t p1 = (size_t)(gpos - options) + 19;
            const size_t p2 = (size_t)(spos - options);
            if (p1 > len) { orc_set_err(err, errcap, "--gaussian_window"); return 1; }
            size_t cnt = (p2 >= p1) ? (p2 - p1) : (len - p1);
            if (cnt > len - p1) cnt = len - p1;
            char buf[256];
            if (cnt >= sizeof(buf)) cnt = sizeof(buf) - 1;
            memcpy(buf, options + p1, cnt);
            buf[cnt] = 0;
            char* end = NULL;
            errno = 0;
            float s = strtof(buf, &end);
            if (end == buf || errno == ERANGE) { orc_set_err(err, errcap, "--gaussian_window"); return 1; }
            if (s > 0) { o->window = ORC_WIN_GAUSSIAN; o->sigma = s; }
        }
    }
    o->remove_dc = strstr(options, "--remove_dc") != NULL;
    o->half_complex = strstr(options, "--half_complex_return") != NULL;
    o->dense = strstr(options, "--layout=dense") != NULL;
    o->serial_power = strstr(options, "--serial_power") != NULL;
    return 0;
}

uint64_t orc_output_floats(const orc_geometry* g, const orc_options* o)
{
    if (!o->dense) return g->ofull;
    const uint64_t bins = (uint64_t)g->n_window / 2 + 1;
    return (uint64_t)g->qt * bins * (o->half_complex ? 2u : 1u);
}

/* ------------------------------------------------------------------ */
/* windows: OKL/kernel.okl:33-127 as translated for the serial runner  */
/* (angle in double stored to float, float cos, double combine)        */
/* ------------------------------------------------------------------ */
float orc_window_value(int kind, int index, int nwin, float sigma)
{
    switch (kind) {
    case ORC_WIN_HANNING: {
        float a = (float)(2.0 * ORC_PI * index / (double)(float)(nwin - 1));
        return (float)(0.5 * (1.0 - (double)cosf(a)));
    }
    case ORC_WIN_HAMMING: {
        float a = (float)(2.0 * ORC_PI * index / (double)(float)(nwin - 1));
        return (float)(0.54 - (0.46 * (double)cosf(a)));
    }
    case ORC_WIN_BLACKMAN: {
        float f = (float)(2.0 * ORC_PI * index / (double)(float)nwin);
        float s = (float)((double)f * 2.0);
        return (float)(0.42 - 0.5 * (double)cosf(f) + 0.08 * (double)cosf(s));
    }
    case ORC_WIN_NUTTALL: {
        float f = (float)(2.0 * ORC_PI * index / (double)(float)nwin);
        float s = (float)((double)f * 2.0);
        float t = (float)((double)f * 3.0);
        return (float)(0.355768 - 0.487396 * (double)cosf(f) + 0.144232 * (double)cosf(s)
                       - 0.012604 * (double)cosf(t));
    }
    case ORC_WIN_BLACKMAN_NUTTALL: {
        float f = (float)(2.0 * ORC_PI * index / (double)(float)nwin);
        float s = (float)((double)f * 2.0);
        float t = (float)((double)f * 3.0);
        return (float)(0.3635819 - 0.4891775 * (double)cosf(f) + 0.1365995 * (double)cosf(s)
                       - 0.0106411 * (double)cosf(t));
    }
    case ORC_WIN_BLACKMAN_HARRIS: {
        float f = (float)(2.0 * ORC_PI * index / (double)(float)nwin);
        float s = (float)((double)f * 2.0);
        float t = (float)((double)f * 3.0);
        return (float)(0.35875 - 0.48829 * (double)cosf(f) + 0.14128 * (double)cosf(s)
                       - 0.01168 * (double)cosf(t));
    }
    case ORC_WIN_FLATTOP: {
        float f = (float)(2.0 * ORC_PI * index / (double)(float)nwin);
        float s = (float)((double)f * 2.0);
        float t = (float)((double)f * 3.0);
        float u = (float)((double)f * 4.0);
        return (float)(0.21557895 - 0.41663158 * (double)cosf(f) + 0.277263158 * (double)cosf(s)
                       - 0.083578947 * (double)cosf(t) + 0.006947368 * (double)cosf(u));
    }
    case ORC_WIN_GAUSSIAN: {
        const int h = nwin >> 1;
        float a = (float)(index - h) / ((float)h * sigma);
        a = a * a;
        a = (float)((double)a * -0.5);
        return expf(a);
    }
    default:
        return 1.0f;
    }
}

/* ------------------------------------------------------------------ */
/* stage restatements                                                  */
/* ------------------------------------------------------------------ */
/* EXPCommon.okl:7-27 */
void orc_overlap(const float* in, uint32_t ofull, uint32_t n, uint32_t exp, uint32_t hop, float* real)
{
    const uint32_t mask = (1u << exp) - 1u;
    for (uint32_t idx = 0; idx < ofull; ++idx) {
        const uint32_t w = idx >> exp;
        const uint32_t l = idx & mask;
        const uint32_t o = w * hop + l;            /* 32-bit, as in the reference */
        const uint32_t ex = o < n;
        real[idx] = in[o * ex] * (float)ex;
    }
}

/* Cost model of the timed CPU baseline.  0 (default): tables built once per
 * call, the fast form for checking.  1: the reference's own per-element work
 * (a window coefficient evaluated for every sample, as Window_* does, and
 * cos/sin of the twiddle angle for every butterfly, as kernel.okl:146-153
 * does), so that the port's time is the reference's time.  The values, and so
 * the outputs, are the same in both modes: each is the same float expression. */
static int g_reference_cost = 0;

void orc_set_reference_cost(int on) { g_reference_cost = on ? 1 : 0; }

/* EXPCommon.okl:29-148 */
void orc_apply_window(int kind, float* data, uint32_t ofull, uint32_t nwin, float sigma, int nthreads)
{
    if (kind == ORC_WIN_NONE) return;
    if (g_reference_cost) {
        const int64_t total = ofull;
#pragma omp parallel for num_threads(nthreads) schedule(static) if (nthreads > 1)
        for (int64_t i = 0; i < total; ++i)
            data[i] *= orc_window_value(kind, (int)((uint64_t)i & (nwin - 1)), (int)nwin, sigma);
        return;
    }
    float* w = (float*)malloc(sizeof(float) * nwin);
    for (uint32_t i = 0; i < nwin; ++i) w[i] = orc_window_value(kind, (int)i, (int)nwin, sigma);
    const int64_t frames = ofull / nwin;
#pragma omp parallel for num_threads(nthreads) schedule(static) if (nthreads > 1)
    for (int64_t f = 0; f < frames; ++f) {
        float* d = data + (uint64_t)f * nwin;
        for (uint32_t i = 0; i < nwin; ++i) d[i] *= w[i];
    }
    free(w);
}

/* EXPCommon.okl:151-192: 64 strided partial sums, then a halving tree */
void orc_remove_dc(float* data, uint32_t ofull, uint32_t nwin, int nthreads)
{
    const int64_t frames = ofull / nwin;
#pragma omp parallel for num_threads(nthreads) schedule(static) if (nthreads > 1)
    for (int64_t f = 0; f < frames; ++f) {
        float* d = data + (uint64_t)f * nwin;
        float added[128];
        for (int i = 0; i < 64; ++i) added[i] = 0.0f;
        for (uint32_t wi = 0; wi < nwin; wi += 64) {
            for (int i = 0; i < 64; ++i) added[i + 64] = d[wi + i];
            for (int i = 0; i < 64; ++i) added[i] += added[i + 64];
        }
        for (unsigned seg = 32; seg > 0; seg >>= 1) {
            for (unsigned i = 0; i < 64; ++i) {
                const unsigned in = i < seg;
                const float l = added[i];
                const float r = added[i + seg];
                added[i] = (l + r) * (float)in;
            }
        }
        const float mean = added[0] / (float)nwin;
        for (uint32_t i = 0; i < nwin; ++i) d[i] -= mean;
    }
}

/* EXPCommon.okl:194-245 with the twiddle of kernel.okl:141-156 */
static void orc_stockham_stage(const float* inR, const float* inI, float* outR, float* outI,
                               uint32_t h, uint32_t stage, uint32_t ohalf, uint32_t exp,
                               int nthreads)
{
    const uint32_t n2 = h << 1;
    const uint32_t seg = 1u << stage;
    /* one twiddle per residue: the same float expression for every frame */
    float* twr = (float*)malloc(sizeof(float) * seg);
    float* twi = (float*)malloc(sizeof(float) * seg);
    for (uint32_t r = 0; r < seg; ++r) {
        const int k = (int)(((int)r * (int)h) / (int)seg);          /* segmentK */
        const float ang = (float)(-2.0 * ORC_PI * (double)((float)k / (float)n2));
        twr[r] = cosf(ang);
        twi[r] = sinf(ang);
    }
    const int64_t frames = ohalf / h;
    if (g_reference_cost) {
        /* the twiddle of every butterfly evaluated where it is used */
#pragma omp parallel for num_threads(nthreads) schedule(static) if (nthreads > 1)
        for (int64_t gi = 0; gi < frames; ++gi) {
            const uint64_t base = (uint64_t)gi * n2;
            for (uint32_t gx = 0; gx < h; ++gx) {
                const uint64_t o = base + gx;
                const float lr = inR[o], li = inI[o];
                const float rr = inR[o + h], ri = inI[o + h];
                const uint64_t ls = (uint64_t)(gx >> stage) * (seg << 1) + (gx & (seg - 1)) + base;
                const uint64_t rs = ls + seg;
                const int k = (int)(((int)(gx & (seg - 1)) * (int)h) / (int)seg);
                const float ang = (float)(-2.0 * ORC_PI * (double)((float)k / (float)n2));
                const float tr = cosf(ang), ti = sinf(ang);
                const float rt = rr * tr - ri * ti;
                const float it = rr * ti + ri * tr;
                outR[ls] = lr + rt;
                outI[ls] = li + it;
                outR[rs] = lr - rt;
                outI[rs] = li - it;
            }
        }
        free(twr);
        free(twi);
        return;
    }
#pragma omp parallel for num_threads(nthreads) schedule(static) if (nthreads > 1)
    for (int64_t gi = 0; gi < frames; ++gi) {
        const uint64_t base = (uint64_t)gi * n2;
        for (uint32_t gx = 0; gx < h; ++gx) {
            const uint64_t o = base + gx;
            const float lr = inR[o], li = inI[o];
            const float rr = inR[o + h], ri = inI[o + h];
            const uint64_t ls = (uint64_t)(gx >> stage) * (seg << 1) + (gx & (seg - 1)) + base;
            const uint64_t rs = ls + seg;
            const uint32_t res = gx & (seg - 1);
            const float tr = twr[res], ti = twi[res];
            const float rt = rr * tr - ri * ti;   /* RMult */
            const float it = rr * ti + ri * tr;   /* IMult */
            outR[ls] = lr + rt;
            outI[ls] = li + it;
            outR[rs] = lr - rt;
            outI[rs] = li - it;
        }
    }
    (void)exp;
    free(twr);
    free(twi);
}

/*
 * Default_Pipeline (RunnerCommon.cpp:184-316) on the Serial runner's buffers
 * (SerialImpl.cpp:47-51).  fix_p4 = 0 reproduces the reference's EXPC result
 * buffer for odd exponents >= 13 (Serial/src/functionImpl.cpp:255-259: the
 * caller keeps reading `real`, which then holds stage exp-2's output).
 */
int orc_serial_pipeline(const float* in, uint32_t n, int exp, float overlap,
                        const char* options, float* out, int fix_p4, int nthreads)
{
    orc_geometry g;
    orc_options o;
    char err[64];
    if (orc_parse_options(options, &o, err, sizeof err)) return 2;
    if (orc_geometry_get(n, exp, overlap, &g)) return 1;
    if (nthreads < 1) nthreads = 1;
    const uint32_t N = g.n_window;
    float* real = (float*)calloc(g.ofull, sizeof(float));
    float* imag = (float*)calloc(g.ofull, sizeof(float));
    float* sreal = (float*)calloc(g.ofull, sizeof(float));
    float* simag = (float*)calloc(g.ofull, sizeof(float));
    if (!real || !imag || !sreal || !simag) {
        free(real); free(imag); free(sreal); free(simag);
        return 3;
    }
    /* Overlap_Common, parallel over 64-sample blocks like the OpenMP runner */
    {
        const int64_t blocks = g.ofull / 64;
        const uint32_t mask = N - 1;
#pragma omp parallel for num_threads(nthreads) schedule(static) if (nthreads > 1)
        for (int64_t b = 0; b < blocks; ++b) {
            for (uint32_t i = 0; i < 64; ++i) {
                const uint32_t idx = (uint32_t)b * 64u + i;
                const uint32_t w = idx >> exp;
                const uint32_t l = idx & mask;
                const uint32_t src = w * g.hop + l;
                const uint32_t ex = src < n;
                real[idx] = in[src * ex] * (float)ex;
            }
        }
    }
    orc_apply_window(o.window, real, g.ofull, N, o.sigma, nthreads);
    if (o.remove_dc) orc_remove_dc(real, g.ofull, N, nthreads);

    /* radix-2 Stockham: stage s reads ping, writes pong */
    const uint32_t h = N >> 1;
    float *aR = real, *aI = imag, *bR = sreal, *bI = simag;
    for (int s = 0; s < exp; ++s) {
        orc_stockham_stage(aR, aI, bR, bI, h, (uint32_t)s, g.ohalf, (uint32_t)exp, nthreads);
        float* t;
        t = aR; aR = bR; bR = t;
        t = aI; aI = bI; bI = t;
    }
    /* aR/aI now hold the full transform.  With exp even it sits in `real`;
     * with exp odd it sits in `sreal`. */
    const float* resR = aR;
    const float* resI = aI;
    if (!fix_p4 && exp >= 12 && (exp & 1)) {
        /* the reference reads `real`, last written by stage exp-2 */
        resR = real;
        resI = imag;
    }
    if (o.half_complex) {
        /* toHalfComplexFormat: ReadIdx == GID, a flat copy of OHalfSize bins */
#pragma omp parallel for num_threads(nthreads) schedule(static) if (nthreads > 1)
        for (int64_t k = 0; k < (int64_t)g.ohalf; ++k) {
            out[2 * k] = resR[k];
            out[2 * k + 1] = resI[k];
        }
    } else {
        /* Serial ToPower passes the real plane twice (functionImpl.cpp:296-301) */
#pragma omp parallel for num_threads(nthreads) schedule(static) if (nthreads > 1)
        for (int64_t k = 0; k < (int64_t)g.ofull; ++k) {
            const float r = resR[k];
            out[k] = sqrtf(r * r + r * r);
        }
    }
    free(real); free(imag); free(sreal); free(simag);
    return 0;
}

/* ------------------------------------------------------------------ */
/* FP64 oracle                                                         */
/* ------------------------------------------------------------------ */
static void orc_fft64(double* re, double* im, uint32_t N, const double* cw, const double* sw)
{
    /* iterative radix-2 DIT, natural order in and out */
    uint32_t j = 0;
    for (uint32_t i = 1; i < N; ++i) {
        uint32_t bit = N >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) {
            double t = re[i]; re[i] = re[j]; re[j] = t;
            t = im[i]; im[i] = im[j]; im[j] = t;
        }
    }
    for (uint32_t len = 2; len <= N; len <<= 1) {
        const uint32_t half = len >> 1;
        const uint32_t step = N / len;
        for (uint32_t b = 0; b < N; b += len) {
            for (uint32_t k = 0; k < half; ++k) {
                const double wr = cw[k * step], wi = sw[k * step];
                const uint32_t p = b + k, q = p + half;
                const double xr = re[q] * wr - im[q] * wi;
                const double xi = re[q] * wi + im[q] * wr;
                re[q] = re[p] - xr;
                im[q] = im[p] - xi;
                re[p] += xr;
                im[p] += xi;
            }
        }
    }
}

int orc_fp64_stft(const float* in, uint32_t n, int exp, float overlap,
                  const char* options, double* out, uint64_t out_cap, int nthreads)
{
    orc_geometry g;
    orc_options o;
    char err[64];
    if (orc_parse_options(options, &o, err, sizeof err)) return 2;
    if (orc_geometry_get(n, exp, overlap, &g)) return 1;
    const uint64_t need = orc_output_floats(&g, &o);
    if (out_cap < need) return 4;
    if (nthreads < 1) nthreads = 1;
    const uint32_t N = g.n_window, M = N / 2;
    double* w = (double*)malloc(sizeof(double) * N);
    double* cw = (double*)malloc(sizeof(double) * N / 2);
    double* sw = (double*)malloc(sizeof(double) * N / 2);
    for (uint32_t i = 0; i < N; ++i)
        w[i] = (double)orc_window_value(o.window, (int)i, (int)N, o.sigma);
    for (uint32_t k = 0; k < N / 2; ++k) {
        const double a = -2.0 * ORC_PI * (double)k / (double)N;
        cw[k] = cos(a);
        sw[k] = sin(a);
    }
    /* compat half-complex only reads the first OHalfSize bins (flat) */
    uint32_t frames = g.qt;
    if (o.half_complex && !o.dense) frames = (uint32_t)(((uint64_t)g.ohalf + N - 1) / N);
#pragma omp parallel num_threads(nthreads) if (nthreads > 1)
    {
        double* re = (double*)malloc(sizeof(double) * N);
        double* im = (double*)malloc(sizeof(double) * N);
#pragma omp for schedule(static)
        for (int64_t f = 0; f < (int64_t)frames; ++f) {
            const uint64_t start = (uint64_t)(uint32_t)((uint32_t)f * g.hop);
            double sum = 0.0;
            for (uint32_t i = 0; i < N; ++i) {
                const uint64_t src = (uint64_t)(uint32_t)(start + i);
                const double x = (src < n) ? (double)in[src] : 0.0;
                re[i] = x * w[i];
                im[i] = 0.0;
                sum += re[i];
            }
            if (o.remove_dc) {
                const double mean = sum / (double)N;
                for (uint32_t i = 0; i < N; ++i) re[i] -= mean;
            }
            orc_fft64(re, im, N, cw, sw);
            if (o.half_complex) {
                if (o.dense) {
                    double* d = out + (uint64_t)f * (M + 1) * 2;
                    for (uint32_t k = 0; k <= M; ++k) { d[2 * k] = re[k]; d[2 * k + 1] = im[k]; }
                } else {
                    const uint64_t base = (uint64_t)f * N;
                    for (uint32_t k = 0; k < N; ++k) {
                        const uint64_t flat = base + k;
                        if (flat >= g.ohalf) break;
                        out[2 * flat] = re[k];
                        out[2 * flat + 1] = im[k];
                    }
                }
            } else {
                const uint32_t nb = o.dense ? M + 1 : N;
                double* d = out + (uint64_t)f * nb;
                for (uint32_t k = 0; k < nb; ++k)
                    d[k] = o.serial_power ? sqrt(2.0) * fabs(re[k]) : hypot(re[k], im[k]);
            }
        }
        free(re);
        free(im);
    }
    free(w); free(cw); free(sw);
    return 0;
}
