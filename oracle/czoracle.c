/*
 * czoracle.c -- CPU oracle for the CubismZ wavelet block codec.
 *
 * TEST INFRASTRUCTURE ONLY (see czoracle.h). Every function restates the
 * reference algorithm and cites the reference file:line it follows. Build
 * with -ffp-contract=off so that double products and sums stay separately
 * rounded, as on x86-64 SSE2 where the reference goldens were produced.
 */
#include "czoracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------ */
/* 4th-order interpolating stencils, evaluated in binary64 and rounded to    */
/* binary32 on return (WaveletsOnInterval.h:33-51: double literals, float    */
/* arguments and return type).                                               */
/* ------------------------------------------------------------------------ */
static float ip_first(float a, float b, float c, float d)
{
    return (float)(5. / 16 * a + 15. / 16 * b - 5. / 16 * c + 1. / 16 * d);
}
static float ip_middle(float a, float b, float c, float d)
{
    return (float)(-1. / 16 * a + 9. / 16 * b + 9. / 16 * c - 1. / 16 * d);
}
static float ip_onetolast(float a, float b, float c, float d)
{
    return (float)(1. / 16 * a - 5. / 16 * b + 15. / 16 * c + 5. / 16 * d);
}
static float ip_last(float a, float b, float c, float d)
{
    return (float)(-5. / 16 * a + 21. / 16 * b - 35. / 16 * c + 35. / 16 * d);
}

/* 3rd-order average-interpolating predictors (WaveletsOnInterval.h:55-83). */
static float p0_first(float a, float b, float c) { return (float)(11. / 8 * a - 1. / 2 * b + 1. / 8 * c); }
static float p1_first(float a, float b, float c) { return (float)(5. / 8 * a + 1. / 2 * b - 1. / 8 * c); }
static float p0_middle(float a, float b, float c) { return (float)(1. / 8 * a + (double)b - 1. / 8 * c); }
static float p1_middle(float a, float b, float c) { return (float)(-1. / 8 * a + (double)b + 1. / 8 * c); }
static float p0_last(float a, float b, float c) { return (float)(-1. / 8 * a + 1. / 2 * b + 5. / 8 * c); }
static float p1_last(float a, float b, float c) { return (float)(1. / 8 * a - 1. / 2 * b + 11. / 8 * c); }

/* WI4::transform<N,forward> (WaveletsOnInterval.h:85-201). Output layout of
 * the forward transform: [N/2 scalings | N/2 details]. */
void czo_transform1d(float *x, int n, int wtype, int fwd)
{
    const int h = n / 2;
    float s[16], d[16];
    int i;
    if (wtype == 1 || wtype == 2) {
        const int lifting = (wtype == 2);
        if (fwd) {
            /* :103-118 details; :120-126 scalings (+ lifting update) */
            d[0] = x[1] - ip_first(x[0], x[2], x[4], x[6]);
            for (i = 1; i < h - 2; ++i)
                d[i] = x[2 * i + 1] - ip_middle(x[2 * i - 2], x[2 * i], x[2 * i + 2], x[2 * i + 4]);
            d[h - 2] = x[n - 3] - ip_onetolast(x[n - 8], x[n - 6], x[n - 4], x[n - 2]);
            d[h - 1] = x[n - 1] - ip_last(x[n - 8], x[n - 6], x[n - 4], x[n - 2]);
            for (i = 0; i < h; ++i) s[i] = x[2 * i];
            if (lifting)
                for (i = 0; i < h; ++i) s[i] = (float)(s[i] + 0.5 * d[i]);
            memcpy(x, s, sizeof(float) * h);
            memcpy(x + h, d, sizeof(float) * h);
        } else {
            /* :131-152 */
            memcpy(s, x, sizeof(float) * h);
            memcpy(d, x + h, sizeof(float) * h);
            if (lifting)
                for (i = 0; i < h; ++i) s[i] = (float)(s[i] - 0.5 * d[i]);
            for (i = 0; i < h; ++i) x[2 * i] = s[i];
            x[1] = ip_first(s[0], s[1], s[2], s[3]) + d[0];
            for (i = 1; i < h - 2; ++i)
                x[2 * i + 1] = ip_middle(s[i - 1], s[i], s[i + 1], s[i + 2]) + d[i];
            x[n - 3] = ip_onetolast(s[h - 4], s[h - 3], s[h - 2], s[h - 1]) + d[h - 2];
            x[n - 1] = ip_last(s[h - 4], s[h - 3], s[h - 2], s[h - 1]) + d[h - 1];
        }
    } else {
        /* wtype 3 and every other value (:154-198) */
        if (fwd) {
            for (i = 0; i < h; ++i) s[i] = (float)(0.5 * (x[2 * i] + x[2 * i + 1]));
            d[0] = (float)(0.5 * ((x[1] - x[0]) - (p1_first(s[0], s[1], s[2]) - p0_first(s[0], s[1], s[2]))));
            for (i = 1; i < h - 1; ++i) {
                const int e = 2 * i;
                d[i] = (float)(0.5 * ((x[e + 1] - x[e]) - (p1_middle(s[i - 1], s[i], s[i + 1]) -
                                                             p0_middle(s[i - 1], s[i], s[i + 1]))));
            }
            d[h - 1] = (float)(0.5 * ((x[n - 1] - x[n - 2]) - (p1_last(s[h - 3], s[h - 2], s[h - 1]) -
                                                               p0_last(s[h - 3], s[h - 2], s[h - 1]))));
            memcpy(x, s, sizeof(float) * h);
            memcpy(x + h, d, sizeof(float) * h);
        } else {
            memcpy(s, x, sizeof(float) * h);
            memcpy(d, x + h, sizeof(float) * h);
            x[0] = p0_first(s[0], s[1], s[2]) - d[0];
            x[1] = p1_first(s[0], s[1], s[2]) + d[0];
            for (i = 1; i < h - 1; ++i) {
                x[2 * i] = p0_middle(s[i - 1], s[i], s[i + 1]) - d[i];
                x[2 * i + 1] = p1_middle(s[i - 1], s[i], s[i + 1]) + d[i];
            }
            x[n - 2] = p0_last(s[h - 3], s[h - 2], s[h - 1]) - d[h - 1];
            x[n - 1] = p1_last(s[h - 3], s[h - 2], s[h - 1]) + d[h - 1];
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Positional sweeps on the [0,bs)^3 corner of a 32^3 array                  */
/* (WaveletSweep, WaveletsOnInterval.h:205-277).                              */
/* ------------------------------------------------------------------------ */
#define AT(b, z, y, x) (b)[((z) * 32 + (y)) * 32 + (x)]

static void rows1d(float *b, int z, int bs, int wtype, int fwd)
{
    for (int y = 0; y < bs; ++y) czo_transform1d(&AT(b, z, y, 0), bs, wtype, fwd);
}
static void xy_swap(float *b, int z, int bs) /* :215-225 */
{
    for (int y = 0; y < bs; ++y)
        for (int x = y + 1; x < bs; ++x) {
            const float t = AT(b, z, y, x);
            AT(b, z, y, x) = AT(b, z, x, y);
            AT(b, z, x, y) = t;
        }
}
static void xz_swap(float *b, int bs) /* :227-238 */
{
    for (int y = 0; y < bs; ++y)
        for (int z = 0; z < bs; ++z)
            for (int x = z + 1; x < bs; ++x) {
                const float t = AT(b, z, y, x);
                AT(b, z, y, x) = AT(b, x, y, z);
                AT(b, x, y, z) = t;
            }
}
static void sweep3d(float *b, int bs, int wtype, int fwd) /* :249-276 */
{
    if (fwd) {
        for (int z = 0; z < bs; ++z) {
            rows1d(b, z, bs, wtype, 1);
            xy_swap(b, z, bs);
            rows1d(b, z, bs, wtype, 1);
        }
        xz_swap(b, bs);
        for (int z = 0; z < bs; ++z) rows1d(b, z, bs, wtype, 1);
    } else {
        for (int z = 0; z < bs; ++z) rows1d(b, z, bs, wtype, 0);
        xz_swap(b, bs);
        for (int z = 0; z < bs; ++z) {
            rows1d(b, z, bs, wtype, 0);
            xy_swap(b, z, bs);
            rows1d(b, z, bs, wtype, 0);
        }
    }
}

/* FullTransformEngine<BS>::fwt/iwt (FullWaveletTransform.h:44-56): levels
 * 32 -> 16 -> 8, the 4^3 base is left untouched (:153-160). */
void czo_fwt(float *block, int wtype)
{
    for (int bs = 32; bs >= 8; bs /= 2) sweep3d(block, bs, wtype, 1);
}
void czo_iwt(float *block, int wtype)
{
    for (int bs = 8; bs <= 32; bs *= 2) sweep3d(block, bs, wtype, 0);
}

/* ------------------------------------------------------------------------ */
/* Thresholding (FullWaveletTransform.h:58-96, base :162-176).               */
/* ------------------------------------------------------------------------ */
int czo_threshold(const float *b, float eps, uint8_t *mask, float *surv)
{
    int n = 0;
    /* coarse 4^3, always kept, z,y,x order */
    for (int z = 0; z < 4; ++z)
        for (int y = 0; y < 4; ++y)
            for (int x = 0; x < 4; ++x) {
                mask[x + 32 * (y + 32 * z)] = 1;
                surv[n++] = AT(b, z, y, x);
            }
    for (int bs = 8; bs <= 32; bs *= 2) {
        const int hh = bs / 2;
        for (int code = 1; code < 8; ++code) {
            const int xs = hh * (code & 1), ys = hh * ((code >> 1) & 1), zs = hh * ((code >> 2) & 1);
            for (int z = 0; z < hh; ++z)
                for (int y = 0; y < hh; ++y)
                    for (int x = 0; x < hh; ++x) {
                        const float v = AT(b, zs + z, ys + y, xs + x);
                        const int keep = fabsf(v) > eps;
                        mask[(xs + x) + 32 * ((ys + y) + 32 * (zs + z))] = (uint8_t)keep;
                        if (keep) surv[n++] = v;
                    }
        }
    }
    return n;
}

/* Inverse of the threshold: FullTransformEngine::load (:99-150, base
 * :178-189). Survivors are consumed from the back in the exact reverse of
 * the push order, so survivor k lands on the k-th kept stream position. */
static void czo_load(float *b, const uint8_t *mask, const float *surv, int n)
{
    int k = n;
    for (int bs = 32; bs >= 8; bs /= 2) {
        const int hh = bs / 2;
        for (int code = 7; code >= 1; --code) {
            const int xs = hh * (code & 1), ys = hh * ((code >> 1) & 1), zs = hh * ((code >> 2) & 1);
            for (int z = hh - 1; z >= 0; --z)
                for (int y = hh - 1; y >= 0; --y)
                    for (int x = hh - 1; x >= 0; --x) {
                        const int eat = mask[(xs + x) + 32 * ((ys + y) + 32 * (zs + z))];
                        AT(b, zs + z, ys + y, xs + x) = eat ? surv[--k] : 0.f;
                    }
        }
    }
    for (int z = 0, c = 0; z < 4; ++z)
        for (int y = 0; y < 4; ++y)
            for (int x = 0; x < 4; ++x, ++c) AT(b, z, y, x) = surv[c];
}

/* ------------------------------------------------------------------------ */
/* Record codec (WaveletCompressor.cpp:33-259).                              */
/* ------------------------------------------------------------------------ */
int czo_block_compress(const float *in, float eps, int wtype, int zerobits, int shuffle,
                       uint8_t *out, int *nbytes)
{
    float *blk = (float *)malloc(sizeof(float) * CZO_BS3);
    uint8_t *mask = (uint8_t *)malloc(CZO_BS3);
    memcpy(blk, in, sizeof(float) * CZO_BS3);
    czo_fwt(blk, wtype);
    float *surv = (float *)(out + CZO_MASKBYTES);
    /* survivors are written straight behind the mask, as at :160 */
    float *tmp = (float *)malloc(sizeof(float) * CZO_BS3);
    const int s = czo_threshold(blk, eps, mask, tmp);
    memcpy(surv, tmp, sizeof(float) * s);
    /* serialize_bitset (:96-122): byte B bit b = mask[8B+b] */
    for (int B = 0; B < CZO_MASKBYTES; ++B) {
        uint8_t c = 0;
        for (int bit = 0; bit < 8; ++bit) c |= (uint8_t)(mask[8 * B + bit] << bit);
        out[B] = c;
    }
    uint8_t *pay = out + CZO_MASKBYTES;
    if (zerobits > 0) { /* float_zero_bits3 (:34-43), applied :166-173 */
        const uint32_t keep = ~((1u << zerobits) - 1u);
        for (int i = 0; i < s; ++i) {
            uint32_t u;
            memcpy(&u, pay + 4 * i, 4);
            u &= keep;
            memcpy(pay + 4 * i, &u, 4);
        }
    }
    if (shuffle && s > 0) { /* shuffle3 (:56-73) with stride 4 */
        const int nb = 4 * s;
        uint8_t *t = (uint8_t *)malloc(nb);
        int j = 0;
        for (int p = 0; p < 4; ++p)
            for (int i = p; i < nb; i += 4) t[j++] = pay[i];
        memcpy(pay, t, nb);
        free(t);
    }
    *nbytes = CZO_MASKBYTES + 4 * s;
    free(tmp);
    free(mask);
    free(blk);
    return 0;
}

int czo_block_decompress(const uint8_t *in, int nbytes, int wtype, int shuffle, float *out)
{
    if (nbytes < CZO_MASKBYTES || nbytes > CZO_MAXRECORD + 4) return -1;
    uint8_t *mask = (uint8_t *)malloc(CZO_BS3);
    int expected = 0; /* deserialize_bitset (:124-150) */
    for (int B = 0; B < CZO_MASKBYTES; ++B)
        for (int bit = 0; bit < 8; ++bit) expected += (mask[8 * B + bit] = (in[B] >> bit) & 1);
    const int nb = nbytes - CZO_MASKBYTES;
    uint8_t *pay = (uint8_t *)malloc(nb > 0 ? nb : 1);
    memcpy(pay, in + CZO_MASKBYTES, nb);
    if (shuffle && nb > 0) { /* reshuffle3 (:75-93) */
        const int c = nb / 4;
        uint8_t *t = (uint8_t *)malloc(nb);
        int j = 0;
        for (int i = 0; i < c; ++i)
            for (int p = 0; p < 4; ++p) t[j++] = pay[i + p * c];
        memcpy(pay, t, (size_t)j);
        free(t);
    }
    int nel = nb / 4; /* :247-251 */
    if (nel - expected == 1) nel--;
    /* the base case consumes exactly the 64 coarse survivors (:178-189), so
     * a well-formed record has every coarse bit set */
    int coarse = 0;
    for (int z = 0; z < 4; ++z)
        for (int y = 0; y < 4; ++y)
            for (int x = 0; x < 4; ++x) coarse += mask[x + 32 * (y + 32 * z)];
    int rc = 0;
    if (nel != expected || coarse != 64) {
        rc = -2;
    } else {
        float *surv = (float *)malloc(sizeof(float) * (nel > 0 ? nel : 1));
        memcpy(surv, pay, sizeof(float) * nel);
        czo_load(out, mask, surv, nel);
        czo_iwt(out, wtype);
        free(surv);
    }
    free(pay);
    free(mask);
    return rc;
}

/* ------------------------------------------------------------------------ */
/* FP64 restatement (quality oracle): the same lifting steps, all binary64.  */
/* ------------------------------------------------------------------------ */
static void t1d_f64(double *x, int n, int wtype, int fwd)
{
    const int h = n / 2;
    double s[16], d[16];
    int i;
#define IF(a, b, c, dd) (5. / 16 * (a) + 15. / 16 * (b) - 5. / 16 * (c) + 1. / 16 * (dd))
#define IM(a, b, c, dd) (-1. / 16 * (a) + 9. / 16 * (b) + 9. / 16 * (c) - 1. / 16 * (dd))
#define IO(a, b, c, dd) (1. / 16 * (a) - 5. / 16 * (b) + 15. / 16 * (c) + 5. / 16 * (dd))
#define IL(a, b, c, dd) (-5. / 16 * (a) + 21. / 16 * (b) - 35. / 16 * (c) + 35. / 16 * (dd))
#define P0F(a, b, c) (11. / 8 * (a) - 1. / 2 * (b) + 1. / 8 * (c))
#define P1F(a, b, c) (5. / 8 * (a) + 1. / 2 * (b) - 1. / 8 * (c))
#define P0M(a, b, c) (1. / 8 * (a) + (b) - 1. / 8 * (c))
#define P1M(a, b, c) (-1. / 8 * (a) + (b) + 1. / 8 * (c))
#define P0L(a, b, c) (-1. / 8 * (a) + 1. / 2 * (b) + 5. / 8 * (c))
#define P1L(a, b, c) (1. / 8 * (a) - 1. / 2 * (b) + 11. / 8 * (c))
    if (wtype == 1 || wtype == 2) {
        const int lifting = (wtype == 2);
        if (fwd) {
            d[0] = x[1] - IF(x[0], x[2], x[4], x[6]);
            for (i = 1; i < h - 2; ++i) d[i] = x[2 * i + 1] - IM(x[2 * i - 2], x[2 * i], x[2 * i + 2], x[2 * i + 4]);
            d[h - 2] = x[n - 3] - IO(x[n - 8], x[n - 6], x[n - 4], x[n - 2]);
            d[h - 1] = x[n - 1] - IL(x[n - 8], x[n - 6], x[n - 4], x[n - 2]);
            for (i = 0; i < h; ++i) s[i] = x[2 * i] + (lifting ? 0.5 * d[i] : 0.);
            memcpy(x, s, sizeof(double) * h);
            memcpy(x + h, d, sizeof(double) * h);
        } else {
            memcpy(s, x, sizeof(double) * h);
            memcpy(d, x + h, sizeof(double) * h);
            if (lifting)
                for (i = 0; i < h; ++i) s[i] -= 0.5 * d[i];
            for (i = 0; i < h; ++i) x[2 * i] = s[i];
            x[1] = IF(s[0], s[1], s[2], s[3]) + d[0];
            for (i = 1; i < h - 2; ++i) x[2 * i + 1] = IM(s[i - 1], s[i], s[i + 1], s[i + 2]) + d[i];
            x[n - 3] = IO(s[h - 4], s[h - 3], s[h - 2], s[h - 1]) + d[h - 2];
            x[n - 1] = IL(s[h - 4], s[h - 3], s[h - 2], s[h - 1]) + d[h - 1];
        }
    } else {
        if (fwd) {
            for (i = 0; i < h; ++i) s[i] = 0.5 * (x[2 * i] + x[2 * i + 1]);
            d[0] = 0.5 * ((x[1] - x[0]) - (P1F(s[0], s[1], s[2]) - P0F(s[0], s[1], s[2])));
            for (i = 1; i < h - 1; ++i)
                d[i] = 0.5 * ((x[2 * i + 1] - x[2 * i]) - (P1M(s[i - 1], s[i], s[i + 1]) - P0M(s[i - 1], s[i], s[i + 1])));
            d[h - 1] = 0.5 * ((x[n - 1] - x[n - 2]) - (P1L(s[h - 3], s[h - 2], s[h - 1]) - P0L(s[h - 3], s[h - 2], s[h - 1])));
            memcpy(x, s, sizeof(double) * h);
            memcpy(x + h, d, sizeof(double) * h);
        } else {
            memcpy(s, x, sizeof(double) * h);
            memcpy(d, x + h, sizeof(double) * h);
            x[0] = P0F(s[0], s[1], s[2]) - d[0];
            x[1] = P1F(s[0], s[1], s[2]) + d[0];
            for (i = 1; i < h - 1; ++i) {
                x[2 * i] = P0M(s[i - 1], s[i], s[i + 1]) - d[i];
                x[2 * i + 1] = P1M(s[i - 1], s[i], s[i + 1]) + d[i];
            }
            x[n - 2] = P0L(s[h - 3], s[h - 2], s[h - 1]) - d[h - 1];
            x[n - 1] = P1L(s[h - 3], s[h - 2], s[h - 1]) + d[h - 1];
        }
    }
}

static void sweep3d_f64(double *b, int bs, int wtype, int fwd)
{
    double t;
    if (fwd) {
        for (int z = 0; z < bs; ++z) {
            for (int y = 0; y < bs; ++y) t1d_f64(&AT(b, z, y, 0), bs, wtype, 1);
            for (int y = 0; y < bs; ++y)
                for (int x = y + 1; x < bs; ++x) { t = AT(b, z, y, x); AT(b, z, y, x) = AT(b, z, x, y); AT(b, z, x, y) = t; }
            for (int y = 0; y < bs; ++y) t1d_f64(&AT(b, z, y, 0), bs, wtype, 1);
        }
        for (int y = 0; y < bs; ++y)
            for (int z = 0; z < bs; ++z)
                for (int x = z + 1; x < bs; ++x) { t = AT(b, z, y, x); AT(b, z, y, x) = AT(b, x, y, z); AT(b, x, y, z) = t; }
        for (int z = 0; z < bs; ++z)
            for (int y = 0; y < bs; ++y) t1d_f64(&AT(b, z, y, 0), bs, wtype, 1);
    } else {
        for (int z = 0; z < bs; ++z)
            for (int y = 0; y < bs; ++y) t1d_f64(&AT(b, z, y, 0), bs, wtype, 0);
        for (int y = 0; y < bs; ++y)
            for (int z = 0; z < bs; ++z)
                for (int x = z + 1; x < bs; ++x) { t = AT(b, z, y, x); AT(b, z, y, x) = AT(b, x, y, z); AT(b, x, y, z) = t; }
        for (int z = 0; z < bs; ++z) {
            for (int y = 0; y < bs; ++y) t1d_f64(&AT(b, z, y, 0), bs, wtype, 0);
            for (int y = 0; y < bs; ++y)
                for (int x = y + 1; x < bs; ++x) { t = AT(b, z, y, x); AT(b, z, y, x) = AT(b, z, x, y); AT(b, z, x, y) = t; }
            for (int y = 0; y < bs; ++y) t1d_f64(&AT(b, z, y, 0), bs, wtype, 0);
        }
    }
}
void czo_fwt_f64(double *block, int wtype)
{
    for (int bs = 32; bs >= 8; bs /= 2) sweep3d_f64(block, bs, wtype, 1);
}
void czo_iwt_f64(double *block, int wtype)
{
    for (int bs = 8; bs <= 32; bs *= 2) sweep3d_f64(block, bs, wtype, 0);
}

/* ------------------------------------------------------------------------ */
/* Adjoint of the inverse transform, from explicit matrices.                 */
/* The inverse line operator of t1d_f64 is linear; M (n x n, row-major,      */
/* out = M in) is built column by column from unit inputs. The 3D adjoint    */
/* runs czo_iwt_f64's steps in reverse order with M^T on every row; the     */
/* xy and xz swaps are their own transposes.                                 */
/* ------------------------------------------------------------------------ */
void czo_inv_matrix(int n, int wtype, double *M)
{
    double e[32];
    for (int j = 0; j < n; ++j) {
        for (int i = 0; i < n; ++i) e[i] = (i == j);
        t1d_f64(e, n, wtype, 0);
        for (int i = 0; i < n; ++i) M[i * n + j] = e[i];
    }
}
static void rows_t(double *b, int z, int bs, const double *M)
{
    double t[32];
    for (int y = 0; y < bs; ++y) {
        double *r = &AT(b, z, y, 0);
        for (int j = 0; j < bs; ++j) {
            double acc = 0;
            for (int i = 0; i < bs; ++i) acc += M[i * bs + j] * r[i];
            t[j] = acc;
        }
        memcpy(r, t, sizeof(double) * bs);
    }
}
void czo_iwt_adj_f64(double *block, int wtype)
{
    double M[32 * 32], t;
    for (int bs = 32; bs >= 8; bs /= 2) {
        czo_inv_matrix(bs, wtype, M);
        for (int z = 0; z < bs; ++z) {
            rows_t(block, z, bs, M);
            for (int y = 0; y < bs; ++y)
                for (int x = y + 1; x < bs; ++x) { t = AT(block, z, y, x); AT(block, z, y, x) = AT(block, z, x, y); AT(block, z, x, y) = t; }
            rows_t(block, z, bs, M);
        }
        for (int y = 0; y < bs; ++y)
            for (int z = 0; z < bs; ++z)
                for (int x = z + 1; x < bs; ++x) { t = AT(block, z, y, x); AT(block, z, y, x) = AT(block, x, y, z); AT(block, x, y, z) = t; }
        for (int z = 0; z < bs; ++z) rows_t(block, z, bs, M);
    }
}

/* ------------------------------------------------------------------------ */
/* LZ4 legacy block format.                                                  */
/* ------------------------------------------------------------------------ */
#define LZ_MINMATCH 4
#define LZ_LASTLIT 5
#define LZ_MFLIMIT 12

int czo_lz4_bound(int isize) { return isize + isize / 255 + 16; } /* lz4.h:81-82 */

/* Decoder restated from LZ4_uncompress_unknownOutputSize (lz4.c:802-905):
 * same acceptance tests, same return convention (-(input position) on
 * error). Deviation: an offset of 0 is rejected (the reference copies
 * unspecified bytes from the output buffer in that case). */
int czo_lz4_decompress(const uint8_t *src, int isize, uint8_t *dst, int cap)
{
    const uint8_t *ip = src, *const iend = src + isize;
    uint8_t *op = dst, *const oend = dst + cap;
    if (ip == iend) return 0; /* :836 goes to the error exit with position 0 */
    for (;;) {
        const unsigned token = *ip++;
        size_t len = token >> 4;
        if (len == 15) {
            int s = 255;
            while (ip < iend && s == 255) { s = *ip++; len += (size_t)s; }
        }
        /* :851: the last sequence holds only literals and ends the input */
        if ((ptrdiff_t)len > oend - op - LZ_MFLIMIT || (ptrdiff_t)len > iend - ip - (2 + 1 + LZ_LASTLIT)) {
            if ((ptrdiff_t)len > oend - op) return -(int)(ip - src);
            if ((ptrdiff_t)len != iend - ip) return -(int)(ip - src);
            memcpy(op, ip, len);
            op += len;
            break;
        }
        memcpy(op, ip, len);
        op += len;
        ip += len;
        const size_t off = (size_t)ip[0] | ((size_t)ip[1] << 8);
        ip += 2;
        if (off == 0 || (ptrdiff_t)off > op - dst) return -(int)(ip - src);
        size_t ml = token & 15;
        if (ml == 15) { /* :873-882 */
            while (ip < iend - (LZ_LASTLIT + 1)) {
                const int s = *ip++;
                ml += (size_t)s;
                if (s == 255) continue;
                break;
            }
        }
        ml += LZ_MINMATCH;
        /* :906-915: a match may not reach into the last 5 output bytes */
        if ((ptrdiff_t)ml > oend - op - LZ_LASTLIT) return -(int)(ip - src);
        const uint8_t *ref = op - off;
        for (size_t k = 0; k < ml; ++k) op[k] = ref[k];
        op += ml;
    }
    return (int)(op - dst);
}

static inline uint32_t rd32(const uint8_t *p)
{
    uint32_t v;
    memcpy(&v, p, 4);
    return v;
}

/* LZ4_compress (lz4.c:695-700) restated: inputs under 65547 bytes take
 * LZ4_compress64kCtx (lz4.c:517-673: 8192-entry table of 16-bit positions,
 * no distance test), larger ones LZ4_compressCtx (lz4.c:337-510: 4096
 * entries, matches at most 65535 back). Both: a zeroed table (every bucket
 * first names position 0), the search starts at position 1, probes advance
 * by attempts >> 6 with attempts starting at 67 at every search, and a
 * probe is made only while the next probe position stays within the
 * match-finder limit; a match extends backwards over equal bytes down to
 * the anchor; after a match the table gets position-2 and the position
 * itself is tested at once (a further match without literals, no backward
 * extension); otherwise the next search starts one byte on. The output is
 * byte for byte the reference's. Returns bytes written (0: cap too small). */
int czo_lz4_compress(const uint8_t *src, int isize, uint8_t *dst, int cap)
{
    const int small = isize < 65536 + LZ_MFLIMIT - 1;
    const int hlog = small ? 13 : 12;
    uint32_t *tab = (uint32_t *)calloc(1u << hlog, sizeof(uint32_t));
    const int mflimit = isize - LZ_MFLIMIT, mlimit = isize - LZ_LASTLIT;
    int ip = 0, anchor = 0;
    uint8_t *op = dst, *const oend = dst + cap;
#define HASHP(p) ((rd32(src + (p)) * 2654435761u) >> (32 - hlog))
#define PUT_LEN(n)                                  \
    do {                                            \
        int r_ = (n);                               \
        for (; r_ >= 255; r_ -= 255) *op++ = 255;   \
        *op++ = (uint8_t)r_;                        \
    } while (0)
    if (isize >= LZ_MFLIMIT + 1) {
        ip = 1;
        uint32_t fwdh = HASHP(ip);
        for (;;) {
            int ref, fwd = ip;
            unsigned attempts = (1u << 6) + 3;
            for (;;) {  /* find a match */
                const uint32_t h = fwdh;
                const int step = (int)(attempts++ >> 6);
                ip = fwd;
                fwd = ip + step;
                if (fwd > mflimit) goto last;
                fwdh = HASHP(fwd);
                ref = (int)tab[h];
                tab[h] = (uint32_t)ip;
                if ((small || ref >= ip - 65535) && rd32(src + ref) == rd32(src + ip)) break;
            }
            while (ip > anchor && ref > 0 && src[ip - 1] == src[ref - 1]) {
                ip--;
                ref--;
            }
            {
                const int lit = ip - anchor;
                if (op + 1 + lit + lit / 255 + 1 + 2 + 8 > oend) { free(tab); return 0; }
                uint8_t *tok = op++;
                if (lit >= 15) {
                    *tok = 15 << 4;
                    PUT_LEN(lit - 15);
                } else {
                    *tok = (uint8_t)(lit << 4);
                }
                memcpy(op, src + anchor, lit);
                op += lit;
                for (;;) {  /* a match at ref for ip; then the position after it */
                    const unsigned off = (unsigned)(ip - ref);
                    *op++ = (uint8_t)off;
                    *op++ = (uint8_t)(off >> 8);
                    int mp = ip + LZ_MINMATCH, rp = ref + LZ_MINMATCH;
                    while (mp < mlimit && src[mp] == src[rp]) { mp++; rp++; }
                    const int ml = mp - ip - LZ_MINMATCH;
                    if (op + 1 + ml / 255 + 1 + LZ_LASTLIT > oend) { free(tab); return 0; }
                    if (ml >= 15) {
                        *tok |= 15;
                        PUT_LEN(ml - 15);
                    } else {
                        *tok |= (uint8_t)ml;
                    }
                    ip = mp;
                    if (ip > mflimit) {
                        anchor = ip;
                        goto last;
                    }
                    tab[HASHP(ip - 2)] = (uint32_t)(ip - 2);
                    const uint32_t h = HASHP(ip);
                    ref = (int)tab[h];
                    tab[h] = (uint32_t)ip;
                    if ((small || ref > ip - 65536) && rd32(src + ref) == rd32(src + ip)) {
                        if (op + 1 + 2 + 8 > oend) { free(tab); return 0; }
                        tok = op++;
                        *tok = 0;
                        continue;
                    }
                    break;
                }
            }
            anchor = ip++;
            fwdh = HASHP(ip);
        }
    }
last: {
    const int lit = isize - anchor;
    if (op + 1 + lit + lit / 255 + 1 > oend) { free(tab); return 0; }
    if (lit >= 15) {
        *op++ = 15 << 4;
        PUT_LEN(lit - 15);
    } else {
        *op++ = (uint8_t)(lit << 4);
    }
    memcpy(op, src + anchor, lit);
    op += lit;
}
#undef PUT_LEN
#undef HASHP
    free(tab);
    return (int)(op - dst);
}

/* ------------------------------------------------------------------------ */
/* Field-level CPU codec (the reference's OpenMP _compress block loop,        */
/* SerializerIO_WaveletCompression_MPI_Simple.h:187-345, with fixed chunking) */
/* ------------------------------------------------------------------------ */
int czo_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

static void gather_block(const float *f, int nx, int ny, int bx, int by, int bz, float *blk)
{
    for (int z = 0; z < 32; ++z)
        for (int y = 0; y < 32; ++y)
            memcpy(blk + (z * 32 + y) * 32, f + ((size_t)(bz * 32 + z) * ny + (by * 32 + y)) * nx + bx * 32,
                   32 * sizeof(float));
}

long long czo_field_compress(const float *field, int nx, int ny, int nz, float eps, int wtype,
                             int zerobits, int shuffle, int encoder, int bpc, int nthreads,
                             uint8_t *out, long long cap, long long *chunk_off)
{
    const int bx = nx / 32, by = ny / 32, bz = nz / 32;
    const int nblocks = bx * by * bz;
    const int nchunks = (nblocks + bpc - 1) / bpc;
    const long long slot = (long long)bpc * (CZO_MAXRECORD + 4);
    const long long zslot = czo_lz4_bound((int)slot);
    uint8_t *stage = (uint8_t *)malloc((size_t)zslot * nchunks);
    long long *csize = (long long *)calloc(nchunks, sizeof(long long));
    int err = 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel
#endif
    {
        float *blk = (float *)malloc(sizeof(float) * CZO_BS3);
        uint8_t *raw = (uint8_t *)malloc((size_t)slot);
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
        for (int c = 0; c < nchunks; ++c) {
            long long used = 0;
            for (int b = c * bpc; b < nblocks && b < (c + 1) * bpc; ++b) {
                const int ix = b % bx, iy = (b / bx) % by, iz = b / (bx * by);
                gather_block(field, nx, ny, ix, iy, iz, blk);
                int nb = 0;
                czo_block_compress(blk, eps, wtype, zerobits, shuffle, raw + used + 4, &nb);
                memcpy(raw + used, &nb, 4);
                used += 4 + nb;
            }
            uint8_t *dst = stage + (size_t)zslot * c;
            if (encoder == 1) {
                const int z = czo_lz4_compress(raw, (int)used, dst, (int)zslot);
                if (z <= 0) err = 1;
                csize[c] = z;
            } else {
                memcpy(dst, raw, (size_t)used);
                csize[c] = used;
            }
        }
        free(raw);
        free(blk);
    }
    long long total = 0;
    for (int c = 0; c < nchunks; ++c) {
        chunk_off[c] = total;
        total += csize[c];
    }
    chunk_off[nchunks] = total;
    if (err || total > cap) {
        free(stage);
        free(csize);
        return -1;
    }
    for (int c = 0; c < nchunks; ++c) memcpy(out + chunk_off[c], stage + (size_t)zslot * c, (size_t)csize[c]);
    free(stage);
    free(csize);
    return total;
}

int czo_field_decompress(const uint8_t *data, const long long *chunk_off, int nchunks, int nx, int ny,
                         int nz, int wtype, int shuffle, int encoder, int bpc, int nthreads, float *field)
{
    const int bx = nx / 32, by = ny / 32, bz = nz / 32;
    const int nblocks = bx * by * bz;
    const long long slot = (long long)bpc * (CZO_MAXRECORD + 4);
    int err = 0;
    (void)nchunks;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel
#endif
    {
        float *blk = (float *)malloc(sizeof(float) * CZO_BS3);
        uint8_t *raw = (uint8_t *)malloc((size_t)slot);
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
        for (int c = 0; c < nchunks; ++c) {
            const uint8_t *src = data + chunk_off[c];
            const int zb = (int)(chunk_off[c + 1] - chunk_off[c]);
            int n;
            if (encoder == 1) {
                n = czo_lz4_decompress(src, zb, raw, (int)slot);
            } else {
                memcpy(raw, src, (size_t)zb);
                n = zb;
            }
            if (n <= 0) { err = 1; continue; }
            int pos = 0;
            for (int b = c * bpc; b < nblocks && b < (c + 1) * bpc; ++b) {
                int nb;
                if (pos + 4 > n) { err = 1; break; }
                memcpy(&nb, raw + pos, 4);
                pos += 4;
                if (nb < 0 || pos + nb > n || czo_block_decompress(raw + pos, nb, wtype, shuffle, blk) != 0) {
                    err = 1;
                    break;
                }
                pos += nb;
                const int ix = b % bx, iy = (b / bx) % by, iz = b / (bx * by);
                for (int z = 0; z < 32; ++z)
                    for (int y = 0; y < 32; ++y)
                        memcpy(field + ((size_t)(iz * 32 + z) * ny + (iy * 32 + y)) * nx + ix * 32,
                               blk + (z * 32 + y) * 32, 32 * sizeof(float));
            }
        }
        free(raw);
        free(blk);
    }
    return err ? -1 : 0;
}
