/*
 * tpal_oracle.c -- CPU oracle for the Transform-PAL hot path.
 *
 * TEST INFRASTRUCTURE, NOT THE PRODUCT: only tests, the smoke check and the
 * benchmark's CPU-baseline leg load this file's library. See tpal_oracle.h
 * for the reference files each part restates. Arithmetic is FP64 in the
 * reference's operation order; build with -ffp-contract=off.
 */
#define _GNU_SOURCE
#include "tpal_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>

#include "fft64.h"

#define MAX_WIDTH 1135 /* PalColour::MAX_WIDTH, src/decoders/palcolour/palcolour.h:93 */

static double dmin(double a, double b) { return (b < a) ? b : a; } /* std::min */
static double dmax(double a, double b) { return (a < b) ? b : a; } /* std::max */
static int32_t imin(int32_t a, int32_t b) { return (b < a) ? b : a; }
static int32_t imax(int32_t a, int32_t b) { return (a < b) ? b : a; }

/* ------------------------------------------------------------------------ */
/* Parameters                                                               */
/* ------------------------------------------------------------------------ */

void tpo_default_params(tpo_params *p, int32_t kind)
{
    memset(p, 0, sizeof(*p));
    /* src/format/video_standards.cpp:58-70,116-207; src/metadata/core.cpp:40-50 */
    p->field_width = 1135;
    p->field_height = 313;
    p->active_start = 177;
    p->active_end = 1125;
    p->first_active_frame_line = 44;
    p->last_active_frame_line = 619;
    p->burst_start = 98;
    p->burst_end = 138;
    p->black = 256 * 64;
    p->white = 844 * 64;
    p->sample_rate = 4.0 * 625.0 * 25.0 * (1135.0 / 4.0 + 1.0 / 625.0);
    p->fsc = 283.75 * 15625.0 + 25.0;
    p->kind = kind;
    p->threshold = 0.4;               /* palcolour.h:73 */
    p->chroma_gain = 1.0;
    p->chroma_phase_deg = 0.0;
    p->output_format = TPO_FMT_P16;
    p->clamp_mode = TPO_CLAMP_NONE;
    p->padding_multiple = 1;
    /* color_conversion.cpp:33-66 at Modern / Scientific */
    p->kb = 0.114;
    p->kr = 0.299;
    p->u_reduction = 0.49211104112248356308804691718185;
    p->v_reduction = 0.87728321993817866838972487283129;
    p->ecb_from_u = 1.0 / ((2.0 * (1.0 - p->kb)) * p->u_reduction);
    p->ecr_from_v = 1.0 / ((2.0 * (1.0 - p->kr)) * p->v_reduction);
    p->y_nr_level = 0.0;
    p->first_field_offset = 0;
    p->sc_locked = 0;
}

/* Field-line range of a field, src/decoders/source_field.h:86-91 */
static int32_t first_active_line(const tpo_params *p, int32_t offset)
{
    return (p->first_active_frame_line + 1 - offset) / 2;
}
static int32_t last_active_line(const tpo_params *p, int32_t offset)
{
    return ((p->last_active_frame_line - offset) / 2) + 1;
}

/* OutputWriter::updateConfiguration geometry, src/output/output_writer.cpp:195-239 */
void tpo_output_geometry(const tpo_params *p, int32_t *width, int32_t *height, int32_t *left_pad, int32_t *top_pad)
{
    const int32_t activeWidth = p->active_end - p->active_start;
    const int32_t activeHeight = (p->last_active_frame_line - p->first_active_frame_line) + 1;
    int32_t lp = 0, rp = 0, tp = 0, bp = 0;
    int32_t ow = activeWidth, oh = activeHeight;
    if (p->padding_multiple > 1) {
        while ((ow % p->padding_multiple) != 0) {
            if ((ow % 2) == 0) rp++;
            else lp++;
            ow = lp + activeWidth + rp;
        }
        while ((oh % p->padding_multiple) != 0) {
            if ((oh % 2) == 0) bp++;
            else tp++;
            oh = tp + activeHeight + bp;
        }
    }
    if (width) *width = ow;
    if (height) *height = oh;
    if (left_pad) *left_pad = lp;
    if (top_pad) *top_pad = tp;
}

size_t tpo_frame_bytes(const tpo_params *p)
{
    int32_t w, h;
    tpo_output_geometry(p, &w, &h, NULL, NULL);
    const size_t planes = (p->output_format == TPO_FMT_GRAY16 || p->output_format == TPO_FMT_GRAYS) ? 1 : 3;
    const size_t bytes = (p->output_format == TPO_FMT_PS || p->output_format == TPO_FMT_RGBS ||
                          p->output_format == TPO_FMT_GRAYS) ? sizeof(float) : sizeof(uint16_t);
    return (size_t)w * (size_t)h * planes * bytes;
}

/* ------------------------------------------------------------------------ */
/* Transform PAL                                                            */
/* ------------------------------------------------------------------------ */

/* transform_pal_2d.cpp:59-62 / transform_pal_3d.cpp:75-78 */
static double compute_window(int32_t element, int32_t limit)
{
    return 0.5 - (0.5 * cos((2 * M_PI * (element + 0.5)) / limit));
}

typedef struct tp_ctx {
    int32_t kind;
    double *window;       /* 2D: 16x32, 3D: 8x32x16 */
    double *thr_sq;       /* 80 or 768 */
    int32_t nthr;
    double *fft_real;
    double *cin, *cout;   /* interleaved complex */
    fft64_plan *plan;
    double *chroma[64];   /* per output field */
    int32_t nchroma;
} tp_ctx;

static int tp_init(tp_ctx *t, const tpo_params *p)
{
    memset(t, 0, sizeof(*t));
    t->kind = p->kind;
    if (p->kind == 1) return 0;   /* PALcolour 2D filter alone: no transform */
    if (p->kind == 2) {
        t->window = (double *)malloc(sizeof(double) * 16 * 32);
        for (int32_t y = 0; y < 16; y++) {
            const double wy = compute_window(y, 16);
            for (int32_t x = 0; x < 32; x++) t->window[y * 32 + x] = wy * compute_window(x, 32);
        }
        t->nthr = 16 * ((17 / 4) + 1); /* getThresholdsSize, transform_pal_2d.cpp:97-101 */
        const int dims[2] = {16, 32};
        t->plan = fft64_plan_create(2, dims);
        t->fft_real = (double *)malloc(sizeof(double) * 512);
        t->cin = (double *)malloc(sizeof(double) * 2 * 16 * 17);
        t->cout = (double *)malloc(sizeof(double) * 2 * 16 * 17);
    } else {
        t->window = (double *)malloc(sizeof(double) * 8 * 32 * 16);
        for (int32_t z = 0; z < 8; z++) {
            const double wz = compute_window(z, 8);
            for (int32_t y = 0; y < 32; y++) {
                const double wy = compute_window(y, 32);
                for (int32_t x = 0; x < 16; x++) t->window[(z * 32 + y) * 16 + x] = wz * wy * compute_window(x, 16);
            }
        }
        t->nthr = 8 * 32 * ((9 / 4) + 1); /* transform_pal_3d.cpp:105-109 */
        const int dims[3] = {8, 32, 16};
        t->plan = fft64_plan_create(3, dims);
        t->fft_real = (double *)malloc(sizeof(double) * 4096);
        t->cin = (double *)malloc(sizeof(double) * 2 * 8 * 32 * 9);
        t->cout = (double *)malloc(sizeof(double) * 2 * 8 * 32 * 9);
    }
    /* TransformPal::updateConfiguration, transform_pal.cpp:53-78 */
    t->thr_sq = (double *)malloc(sizeof(double) * t->nthr);
    if (p->thresholds == NULL || p->n_thresholds == 0) {
        for (int32_t i = 0; i < t->nthr; i++) t->thr_sq[i] = p->threshold * p->threshold;
    } else {
        if (p->n_thresholds != t->nthr) return -1;
        for (int32_t i = 0; i < t->nthr; i++) t->thr_sq[i] = p->thresholds[i] * p->thresholds[i];
    }
    return (t->plan && t->window && t->fft_real && t->cin && t->cout) ? 0 : -1;
}

static void tp_free(tp_ctx *t)
{
    free(t->window);
    free(t->thr_sq);
    free(t->fft_real);
    free(t->cin);
    free(t->cout);
    fft64_plan_destroy(t->plan);
    for (int32_t i = 0; i < t->nchroma; i++) free(t->chroma[i]);
}

static double abs_sq(const double *c) { return (c[0] * c[0]) + (c[1] * c[1]); }

/* TransformPal2D::applyFilter, transform_pal_2d.cpp:210-287 */
static void apply_filter_2d(tp_ctx *t)
{
    const int XC = 17;
    const double *thr = t->thr_sq;
    memset(t->cout, 0, sizeof(double) * 2 * 16 * XC);
    for (int32_t y = 0; y < 16; y++) {
        const int32_t y_ref = ((16 / 2) + 16 - y) % 16;
        const double *bi = t->cin + 2 * (y * XC);
        const double *bi_ref = t->cin + 2 * (y_ref * XC);
        double *bo = t->cout + 2 * (y * XC);
        double *bo_ref = t->cout + 2 * (y_ref * XC);
        for (int32_t x = 32 / 8; x <= 32 / 4; x++) {
            const int32_t x_ref = (32 / 2) - x;
            const double threshold_sq = *thr++;
            const double *in_val = bi + 2 * x;
            const double *ref_val = bi_ref + 2 * x_ref;
            if (x == x_ref && y == y_ref) {
                bo[2 * x] = in_val[0];
                bo[2 * x + 1] = in_val[1];
                continue;
            }
            const double m_in_sq = abs_sq(in_val);
            const double m_ref_sq = abs_sq(ref_val);
            if (m_in_sq < m_ref_sq * threshold_sq || m_ref_sq < m_in_sq * threshold_sq) {
            } else {
                bo[2 * x] = in_val[0];
                bo[2 * x + 1] = in_val[1];
                bo_ref[2 * x_ref] = ref_val[0];
                bo_ref[2 * x_ref + 1] = ref_val[1];
            }
        }
    }
}

/* TransformPal3D::applyFilter, transform_pal_3d.cpp:249-333 */
static void apply_filter_3d(tp_ctx *t)
{
    const int XC = 9, YC = 32;
    const double *thr = t->thr_sq;
    memset(t->cout, 0, sizeof(double) * 2 * 8 * YC * XC);
    for (int32_t z = 0; z < 8; z++) {
        const int32_t z_ref = ((8 / 4) + 8 - z) % 8;
        for (int32_t y = 0; y < 32; y++) {
            const int32_t y_ref = ((32 / 4) + 32 - y) % 32;
            const double *bi = t->cin + 2 * ((z * YC + y) * XC);
            const double *bi_ref = t->cin + 2 * ((z_ref * YC + y_ref) * XC);
            double *bo = t->cout + 2 * ((z * YC + y) * XC);
            double *bo_ref = t->cout + 2 * ((z_ref * YC + y_ref) * XC);
            for (int32_t x = 16 / 8; x <= 16 / 4; x++) {
                const int32_t x_ref = (16 / 2) - x;
                const double threshold_sq = *thr++;
                const double *in_val = bi + 2 * x;
                const double *ref_val = bi_ref + 2 * x_ref;
                if (x == x_ref && y == y_ref && z == z_ref) {
                    bo[2 * x] = in_val[0];
                    bo[2 * x + 1] = in_val[1];
                    continue;
                }
                const double m_in_sq = abs_sq(in_val);
                const double m_ref_sq = abs_sq(ref_val);
                if (m_in_sq < m_ref_sq * threshold_sq || m_ref_sq < m_in_sq * threshold_sq) {
                } else {
                    bo[2 * x] = in_val[0];
                    bo[2 * x + 1] = in_val[1];
                    bo_ref[2 * x_ref] = ref_val[0];
                    bo_ref[2 * x_ref + 1] = ref_val[1];
                }
            }
        }
    }
}

typedef struct src_field {
    const uint16_t *data;
    int32_t offset; /* 0 first field, 1 second */
} src_field;

/* TransformPal2D::filterField, transform_pal_2d.cpp:133-200 */
static void filter_field_2d(tp_ctx *t, const tpo_params *p, const src_field *f, double *out)
{
    const int32_t fw = p->field_width;
    const int32_t firstFieldLine = first_active_line(p, f->offset);
    const int32_t lastFieldLine = last_active_line(p, f->offset);
    for (int32_t tileY = firstFieldLine - 8; tileY < lastFieldLine; tileY += 8) {
        const int32_t startY = imax(firstFieldLine - tileY, 0);
        const int32_t endY = imin(lastFieldLine - tileY, 16);
        for (int32_t tileX = p->active_start - 16; tileX < p->active_end; tileX += 16) {
            for (int32_t y = 0; y < 16; y++) {
                if (y < startY || y >= endY) {
                    for (int32_t x = 0; x < 32; x++) t->fft_real[y * 32 + x] = p->black * t->window[y * 32 + x];
                    continue;
                }
                const uint16_t *b = f->data + ((tileY + y) * fw);
                for (int32_t x = 0; x < 32; x++) t->fft_real[y * 32 + x] = b[tileX + x] * t->window[y * 32 + x];
            }
            fft64_r2c(t->plan, t->fft_real, t->cin);
            apply_filter_2d(t);
            const int32_t startX = imax(p->active_start - tileX, 0);
            const int32_t endX = imin(p->active_end - tileX, 32);
            fft64_c2r(t->plan, t->cout, t->fft_real);
            for (int32_t y = startY; y < endY; y++) {
                double *b = out + ((tileY + y) * fw);
                for (int32_t x = startX; x < endX; x++) b[tileX + x] += t->fft_real[y * 32 + x] / (16 * 32);
            }
        }
    }
}

/* TransformPal3D::filterFields, transform_pal_3d.cpp:123-240 */
static void filter_fields_3d(tp_ctx *t, const tpo_params *p, const src_field *fields, int32_t startIndex,
                             int32_t endIndex, double **out)
{
    const int32_t fw = p->field_width;
    for (int32_t tileZ = startIndex - 4; tileZ < endIndex; tileZ += 4) {
        for (int32_t tileY = p->first_active_frame_line - 16; tileY <= p->last_active_frame_line; tileY += 16) {
            for (int32_t tileX = p->active_start - 8; tileX < p->active_end; tileX += 8) {
                const int32_t startY = imax(p->first_active_frame_line - tileY, 0);
                const int32_t endY = imin((p->last_active_frame_line - tileY) + 1, 32);
                for (int32_t z = 0; z < 8; z++) {
                    const int32_t fieldIndex = tileZ + z;
                    const int32_t fieldOffset = fields[fieldIndex].offset;
                    const uint16_t *inputPtr = fields[fieldIndex].data;
                    for (int32_t y = 0; y < 32; y++) {
                        double *dst = t->fft_real + (z * 32 + y) * 16;
                        const double *w = t->window + (z * 32 + y) * 16;
                        if (y < startY || y >= endY || ((tileY + y) % 2) != fieldOffset) {
                            for (int32_t x = 0; x < 16; x++) dst[x] = p->black * w[x];
                            continue;
                        }
                        const int32_t fieldLine = (tileY + y) / 2;
                        const uint16_t *b = inputPtr + (fieldLine * fw);
                        for (int32_t x = 0; x < 16; x++) dst[x] = b[tileX + x] * w[x];
                    }
                }
                fft64_r2c(t->plan, t->fft_real, t->cin);
                apply_filter_3d(t);
                const int32_t startX = imax(p->active_start - tileX, 0);
                const int32_t endX = imin(p->active_end - tileX, 16);
                const int32_t startZ = imax(startIndex - tileZ, 0);
                const int32_t endZ = imin(endIndex - tileZ, 8);
                fft64_c2r(t->plan, t->cout, t->fft_real);
                for (int32_t z = startZ; z < endZ; z++) {
                    const int32_t fieldIndex = tileZ + z;
                    const int32_t fieldOffset = fields[fieldIndex].offset;
                    double *outputPtr = out[fieldIndex - startIndex];
                    for (int32_t y = startY; y < endY; y++) {
                        if (((tileY + y) % 2) != fieldOffset) continue;
                        const int32_t outputLine = (tileY + y) / 2;
                        double *b = outputPtr + (outputLine * fw);
                        for (int32_t x = startX; x < endX; x++)
                            b[tileX + x] += t->fft_real[((z * 32) + y) * 16 + x] / (8 * 32 * 16);
                    }
                }
            }
        }
    }
}

/* ------------------------------------------------------------------------ */
/* PALcolour demodulator                                                    */
/* ------------------------------------------------------------------------ */

typedef struct pal_ctx {
    double sine[MAX_WIDTH], cosine[MAX_WIDTH];
    int32_t filterSize;
    double cfilt[64][4];
    double yfilt[64][2];
} pal_ctx;

/* PalColour::buildLookUpTables, palcolour.cpp:150-277 */
static void pal_build(pal_ctx *c, const tpo_params *p)
{
    if (p->field_height != 263) {
        for (int32_t i = 0; i < p->field_width; i++) {
            const double rad = 2 * M_PI * i * p->fsc / p->sample_rate;
            c->sine[i] = sin(rad);
            c->cosine[i] = cos(rad);
        }
    } else {
        for (int32_t i = 0; i < p->field_width; i++) {
            const double rad = 2 * M_PI * i * p->fsc / p->sample_rate;
            c->sine[i] = cos(rad);
            c->cosine[i] = sin(rad);
        }
    }
    const double chromaBandwidthHz = 1100000.0 / 0.93;
    const double ca = 0.5 * p->sample_rate / chromaBandwidthHz;
    const double ya = 0.5 * p->sample_rate / chromaBandwidthHz;
    int32_t fs = 1;
    if ((int32_t)ca > fs) fs = (int32_t)ca;
    if ((int32_t)ya > fs) fs = (int32_t)ya;
    if (fs > 63) fs = 63;
    c->filterSize = fs;
    double cdiv = 0, ydiv = 0;
    for (int32_t f = 0; f <= fs; f++) {
        const double fc = dmin(ca, (double)f);
        const double ff = dmin(ca, sqrt(f * f + 2 * 2));
        const double fff = dmin(ca, sqrt(f * f + 4 * 4));
        const double ffff = dmin(ca, sqrt(f * f + 6 * 6));
        const int32_t d = (f == 0) ? 2 : 1;
        c->cfilt[f][0] = (1 + cos(M_PI * fc / ca)) / d;
        c->cfilt[f][2] = (1 + cos(M_PI * ff / ca)) / d;
        c->cfilt[f][1] = (1 + cos(M_PI * fff / ca)) / d;
        c->cfilt[f][3] = (1 + cos(M_PI * ffff / ca)) / d;
        cdiv += 2 * (1 * c->cfilt[f][0] + 2 * c->cfilt[f][2] + 2 * c->cfilt[f][1] + 2 * c->cfilt[f][3]);
        const double fy = dmin(ya, (double)f);
        const double fffy = dmin(ya, sqrt(f * f + 4 * 4));
        c->yfilt[f][0] = (1 + cos(M_PI * fy / ya)) / d;
        c->yfilt[f][1] = 0.2 * (1 + cos(M_PI * fffy / ya)) / d;
        ydiv += 2 * (1 * c->yfilt[f][0] + 2 * 0 + 2 * c->yfilt[f][1] + 2 * 0);
    }
    for (int32_t f = 0; f <= fs; f++) {
        for (int32_t i = 0; i < 4; i++) c->cfilt[f][i] /= cdiv;
        for (int32_t i = 0; i < 2; i++) c->yfilt[f][i] /= ydiv;
    }
}

typedef struct line_info {
    int32_t number;
    double bp, bq, Vsw;
} line_info;

static const uint16_t kBlackLine16[MAX_WIDTH];  /* zeros */
static const double kBlackLineD[MAX_WIDTH];     /* zeros */

/* PalColour::detectBurst, palcolour.cpp:344-409 */
static void detect_burst(const pal_ctx *c, const tpo_params *p, line_info *line, const uint16_t *inputData)
{
    const int32_t fw = p->field_width, fh = p->field_height;
    const uint16_t *in0 = inputData + (line->number * fw);
    const uint16_t *in1 = (line->number - 1) < 0 ? kBlackLine16 : (inputData + ((line->number - 1) * fw));
    const uint16_t *in2 = (line->number + 1) >= fh ? kBlackLine16 : (inputData + ((line->number + 1) * fw));
    const uint16_t *in3 = (line->number - 2) < 0 ? kBlackLine16 : (inputData + ((line->number - 2) * fw));
    const uint16_t *in4 = (line->number + 2) >= fh ? kBlackLine16 : (inputData + ((line->number + 2) * fw));
    double bp = 0, bq = 0, bpo = 0, bqo = 0;
    for (int32_t i = p->burst_start; i < p->burst_end; i++) {
        bp += ((in0[i] - ((in3[i] + in4[i]) / 2.0)) / 2.0) * c->sine[i];
        bq += ((in0[i] - ((in3[i] + in4[i]) / 2.0)) / 2.0) * c->cosine[i];
        bpo += ((in2[i] - in1[i]) / 2.0) * c->sine[i];
        bqo += ((in2[i] - in1[i]) / 2.0) * c->cosine[i];
    }
    const int32_t colourBurstLength = p->burst_end - p->burst_start;
    bp /= colourBurstLength;
    bq /= colourBurstLength;
    bpo /= colourBurstLength;
    bqo /= colourBurstLength;
    line->Vsw = -1;
    if ((((bp - bpo) * (bp - bpo) + (bq - bqo) * (bq - bqo)) < (bp * bp + bq * bq) * 2)) line->Vsw = 1;
    line->bp = (bp - bqo) / 2;
    line->bq = (bq + bpo) / 2;
    const double burstNorm = dmax(sqrt(line->bp * line->bp + line->bq * line->bq), 130000.0 / 128);
    line->bp /= burstNorm;
    line->bq /= burstNorm;
}

typedef struct component_frame {
    int32_t width, height;
    double *y, *u, *v;
} component_frame;

/* The 25-tap high-pass of doYNR, c_nrpal_b (src/decoders/filter/deemp.h:620-628). */
static const double kNrPal[25] = {
    1.141291975113614e-04, -1.857019211291029e-03, -4.499636864042073e-03, -5.577680979937061e-03,
    -4.423694440267179e-04, 1.309163063177155e-02, 2.861211356202848e-02, 3.029931283148555e-02,
    1.098965697652802e-03, -6.398130386469833e-02, -1.492080690537196e-01, -2.223459379380252e-01,
    7.479077367478024e-01, -2.223459379380252e-01, -1.492080690537196e-01, -6.398130386469833e-02,
    1.098965697652803e-03, 3.029931283148557e-02, 2.861211356202848e-02, 1.309163063177156e-02,
    -4.423694440267185e-04, -5.577680979937061e-03, -4.499636864042074e-03, -1.857019211291030e-03,
    1.141291975113614e-04};

/* PalColour::doYNR, palcolour.cpp:412-449, with IIRFilter<25,1>::feed
 * (src/decoders/filter/iirfilter.h:69-83): output = b0*x[t] then b[i]*x[t-i]
 * for i = 24 down to 1; zeros fed before and after the active samples. */
static void do_ynr(const tpo_params *p, double *Yline, double *hist, double *hpY)
{
    const double irescale = (double)((p->white - p->black) / 100);   /* integer division, as the reference */
    const double nr_y = p->y_nr_level * irescale;
    const int32_t delay = 25 / 2;
    for (int32_t i = 0; i < 25; i++) hist[i] = 0.0;
    /* feed(v): y0 = b0*v + sum_{i=24..1} b[i]*x[i] (x shifted first) */
#define YNR_FEED(v, outv)                                              \
    do {                                                               \
        double y0 = kNrPal[0] * (v);                                   \
        for (int32_t i = 24; i >= 1; i--) {                            \
            hist[i] = hist[i - 1];                                     \
            y0 += kNrPal[i] * hist[i];                                 \
        }                                                              \
        hist[0] = (v);                                                 \
        outv = y0;                                                     \
    } while (0)
    double sink;
    for (int32_t h = p->active_start - delay; h < p->active_start; h++) YNR_FEED(0.0, sink);
    (void)sink;
    for (int32_t h = p->active_start; h < p->active_end; h++) YNR_FEED(Yline[h], hpY[h]);
    for (int32_t h = p->active_end; h < p->active_end + delay; h++) YNR_FEED(0.0, hpY[h]);
#undef YNR_FEED
    for (int32_t h = p->active_start; h < p->active_end; h++) {
        double a = hpY[h + delay];
        if (fabs(a) > nr_y) a = (a > 0) ? nr_y : -nr_y;
        Yline[h] -= a;
    }
}

/* PalColour::decodeLine, palcolour.cpp:456-646: decodeLine<double, true> on
 * Transform-PAL chroma (kinds 2, 3) and decodeLine<uint16_t, false> on the
 * composite (kind 1, the PALcolour 2D filter with luma resynthesised from
 * the Y filter). simplePAL is not reachable from the ABI. */
static void decode_line(const pal_ctx *c, const tpo_params *p, const src_field *f, const double *chromaData,
                        const line_info *line, component_frame *cf, double (*m)[MAX_WIDTH],
                        double (*n)[MAX_WIDTH], double *pu, double *qu, double *pv, double *qv, double *py,
                        double *qy, double *scratch)
{
    const int32_t fw = p->field_width;
    const int32_t firstLine = first_active_line(p, f->offset);
    const int32_t lastLine = last_active_line(p, f->offset);
    const int prefiltered = (p->kind != 1);
    /* input rows as doubles: chroma for the transform kinds, composite for kind 1 (blackLine = 0) */
    const double *rows[7];
    const int32_t dl[7] = {0, -1, 1, -2, 2, -3, 3};
    double *tmp = scratch;   /* 7 rows of MAX_WIDTH for the composite case */
    for (int r = 0; r < 7; r++) {
        const int32_t ln = line->number + dl[r];
        const int outside = (r == 0) ? 0 : ((dl[r] < 0) ? (ln < firstLine) : (ln >= lastLine));
        if (outside) {
            rows[r] = kBlackLineD;
        } else if (prefiltered) {
            rows[r] = chromaData + (ln * fw);
        } else {
            const uint16_t *src = f->data + (ln * fw);
            double *d = tmp + (size_t)r * MAX_WIDTH;
            for (int32_t i = 0; i < fw; i++) d[i] = src[i];
            rows[r] = d;
        }
    }
    const double *in0 = rows[0], *in1 = rows[1], *in2 = rows[2], *in3 = rows[3], *in4 = rows[4], *in5 = rows[5],
                 *in6 = rows[6];
    const int32_t endPos = imin(p->active_end, MAX_WIDTH);
    const int32_t filterSize = c->filterSize;
    const int32_t fillStart = imax(0, p->active_start - filterSize);
    const int32_t fillEnd = imin(p->active_end + filterSize + 1, MAX_WIDTH);
    const double *sine = c->sine, *cosine = c->cosine;
    for (int32_t i = fillStart; i < fillEnd; i++) {
        m[0][i] = in0[i] * sine[i];
        m[2][i] = in1[i] * sine[i] - in2[i] * sine[i];
        m[1][i] = -in3[i] * sine[i] - in4[i] * sine[i];
        m[3][i] = -in5[i] * sine[i] + in6[i] * sine[i];
        n[0][i] = in0[i] * cosine[i];
        n[2][i] = in1[i] * cosine[i] - in2[i] * cosine[i];
        n[1][i] = -in3[i] * cosine[i] - in4[i] * cosine[i];
        n[3][i] = -in5[i] * cosine[i] + in6[i] * cosine[i];
    }
    for (int32_t i = p->active_start; i < endPos; i++) {
        double PU = 0, QU = 0, PV = 0, QV = 0, PY = 0, QY = 0;
        for (int32_t b = 0; b <= filterSize; b++) {
            const int32_t l = imax(fillStart, i - b);
            const int32_t r = imin(fillEnd - 1, i + b);
            const double *cf4 = c->cfilt[b];
            PY += (m[0][r] + m[0][l]) * c->yfilt[b][0] + (m[1][r] + m[1][l]) * c->yfilt[b][1];
            QY += (n[0][r] + n[0][l]) * c->yfilt[b][0] + (n[1][r] + n[1][l]) * c->yfilt[b][1];
            PU += (m[0][r] + m[0][l]) * cf4[0] + (m[1][r] + m[1][l]) * cf4[1] + (n[2][r] + n[2][l]) * cf4[2] +
                  (n[3][r] + n[3][l]) * cf4[3];
            QU += (n[0][r] + n[0][l]) * cf4[0] + (n[1][r] + n[1][l]) * cf4[1] - (m[2][r] + m[2][l]) * cf4[2] -
                  (m[3][r] + m[3][l]) * cf4[3];
            PV += (m[0][r] + m[0][l]) * cf4[0] + (m[1][r] + m[1][l]) * cf4[1] - (n[2][r] + n[2][l]) * cf4[2] -
                  (n[3][r] + n[3][l]) * cf4[3];
            QV += (n[0][r] + n[0][l]) * cf4[0] + (n[1][r] + n[1][l]) * cf4[1] + (m[2][r] + m[2][l]) * cf4[2] +
                  (m[3][r] + m[3][l]) * cf4[3];
        }
        pu[i] = PU;
        qu[i] = QU;
        pv[i] = PV;
        qv[i] = QV;
        py[i] = PY;
        qy[i] = QY;
    }
    const uint16_t *comp = f->data + (line->number * fw);
    const int32_t lineNumber = (line->number * 2) + f->offset;
    double *outY = cf->y + (size_t)lineNumber * cf->width;
    double *outU = cf->u + (size_t)lineNumber * cf->width;
    double *outV = cf->v + (size_t)lineNumber * cf->width;
    for (int32_t i = p->active_start; i < endPos; i++) {
        if (prefiltered) outY[i] = comp[i] - in0[i];
        else outY[i] = comp[i] - ((py[i] * sine[i] + qy[i] * cosine[i]) * 2.0);
        outU[i] = -(pu[i] * line->bp + qu[i] * line->bq) * 2.0;
        outV[i] = line->Vsw * -(qv[i] * line->bp - pv[i] * line->bq) * 2.0;
    }
    if (p->y_nr_level > 0.0) do_ynr(p, outY, scratch + 7 * (size_t)MAX_WIDTH, scratch + 8 * (size_t)MAX_WIDTH);
}

typedef struct demod_scratch {
    double m[4][MAX_WIDTH], n[4][MAX_WIDTH];
    double pu[MAX_WIDTH], qu[MAX_WIDTH], pv[MAX_WIDTH], qv[MAX_WIDTH], py[MAX_WIDTH], qy[MAX_WIDTH];
    double rows[9 * MAX_WIDTH + 64];   /* composite rows, yNR history and high-pass output */
} demod_scratch;

/* PalColour::decodeField, palcolour.cpp:307-335 */
static void decode_field(const pal_ctx *c, const tpo_params *p, const src_field *f, const double *chroma,
                         component_frame *cf, demod_scratch *s)
{
    const int32_t firstLine = first_active_line(p, f->offset);
    const int32_t lastLine = last_active_line(p, f->offset);
    for (int32_t fieldLine = firstLine; fieldLine < lastLine; fieldLine++) {
        line_info line;
        line.number = fieldLine;
        detect_burst(c, p, &line, f->data);
        const double oldBp = line.bp, oldBq = line.bq;
        const double theta = (p->chroma_phase_deg * M_PI) / 180;
        line.bp = (oldBp * cos(theta) - oldBq * sin(theta)) * p->chroma_gain;
        line.bq = (oldBp * sin(theta) + oldBq * cos(theta)) * p->chroma_gain;
        decode_line(c, p, f, chroma, &line, cf, s->m, s->n, s->pu, s->qu, s->pv, s->qv, s->py, s->qy, s->rows);
    }
}

/* ------------------------------------------------------------------------ */
/* Output writer                                                            */
/* ------------------------------------------------------------------------ */

/* output_writer.cpp:60-76 */
static double h273_round(double x) { return (x < 0.0 ? -1.0 : 1.0) * floor(fabs(x) + 0.5); }
static double dclamp(double v, double lo, double hi) { return (v < lo) ? lo : ((hi < v) ? hi : v); }
static float fclamp(float v, float lo, float hi) { return (v < lo) ? lo : ((hi < v) ? hi : v); }

/* intYCbCrBounds / floatYCbCrBounds, output_writer.cpp:84-143 */
static void int_bounds(int32_t mode, double *b)
{
    switch (mode) {
    case TPO_CLAMP_LEGAL_RGB_SDR:
        b[0] = 16.0 * 256.0; b[1] = 235.0 * 256.0; b[2] = 16.0 * 256.0; b[3] = 240.0 * 256.0;
        break;
    case TPO_CLAMP_LEGAL_YCBCR_BT601:
        b[0] = 1.0 * 256.0; b[1] = 254.75 * 256.0; b[2] = 1.0 * 256.0; b[3] = 254.75 * 256.0;
        break;
    default:
        b[0] = 0.0; b[1] = 65535.0; b[2] = 0.0; b[3] = 65535.0;
    }
}
static void float_bounds(int32_t mode, float *b)
{
    switch (mode) {
    case TPO_CLAMP_LEGAL_RGB_SDR:
        b[0] = 0.0f; b[1] = 1.0f; b[2] = -0.5f; b[3] = 0.5f;
        break;
    case TPO_CLAMP_LEGAL_YCBCR_BT601:
        b[0] = -15.0f / 219.0f; b[1] = 238.75f / 219.0f; b[2] = -127.0f / 224.0f; b[3] = 126.75f / 224.0f;
        break;
    default:
        b[0] = -INFINITY; b[1] = INFINITY; b[2] = -INFINITY; b[3] = INFINITY;
    }
}

/* floatRGBBounds, output_writer.cpp:149-190 */
static void float_rgb_bounds(const tpo_params *p, float *b)
{
    const float inf = INFINITY;
    switch (p->clamp_mode) {
    case TPO_CLAMP_LEGAL_RGB_SDR:
        for (int i = 0; i < 3; i++) { b[2 * i] = 0.0f; b[2 * i + 1] = 1.0f; }
        break;
    case TPO_CLAMP_LEGAL_RGB_HDR:
        for (int i = 0; i < 3; i++) { b[2 * i] = 0.0f; b[2 * i + 1] = inf; }
        break;
    case TPO_CLAMP_LEGAL_YCBCR_BT601: {
        float yb[4];
        float_bounds(p->clamp_mode, yb);
        const double kg = 1.0 - p->kr - p->kb;
        const double bds = 2.0 * (1.0 - p->kb), rds = 2.0 * (1.0 - p->kr);
        const double gFromCb = (p->kb * bds) / kg;
        const double gFromCr = (p->kr * rds) / kg;
        b[0] = (float)(yb[0] + rds * yb[2]);
        b[1] = (float)(yb[1] + rds * yb[3]);
        b[2] = (float)(yb[0] - (gFromCb + gFromCr) * yb[3]);
        b[3] = (float)(yb[1] - (gFromCb + gFromCr) * yb[2]);
        b[4] = (float)(yb[0] + bds * yb[2]);
        b[5] = (float)(yb[1] + bds * yb[3]);
        break;
    }
    default:
        for (int i = 0; i < 3; i++) { b[2 * i] = -inf; b[2 * i + 1] = inf; }
    }
}

/* OutputWriter::convert / convertLine (YUV444P16, RGB48, GRAY16),
 * convertToFloat (YUV444PS, GRAYS) and convertToFloatRGB (RGBS),
 * output_writer.cpp:340-486, 670-779, with ColorConversion's derived
 * scalars (color_conversion.cpp:33-66). */
static void write_output(const tpo_params *p, const component_frame *cf, void *out)
{
    int32_t ow, oh, lp, tpad;
    tpo_output_geometry(p, &ow, &oh, &lp, &tpad);
    const int32_t activeWidth = p->active_end - p->active_start;
    const int32_t activeHeight = (p->last_active_frame_line - p->first_active_frame_line) + 1;
    const size_t planeSize = (size_t)ow * oh;
    const double yOffset = p->black;
    const double yRange = p->white - p->black;
    const double uvRange = yRange;
    const double eyScale = 1.0 / yRange;
    const double ecbScale = p->ecb_from_u / uvRange;
    const double ecrScale = p->ecr_from_v / uvRange;
    const double kg = 1.0 - p->kr - p->kb;
    const double rFromV = 1.0 / p->v_reduction;
    const double gFromU = -(p->kb / kg) / p->u_reduction;
    const double gFromV = -(p->kr / kg) / p->v_reduction;
    const double bFromU = 1.0 / p->u_reduction;
    const int32_t fmt = p->output_format;
    const int padded = (ow != activeWidth || oh != activeHeight);
    if (fmt == TPO_FMT_PS || fmt == TPO_FMT_GRAYS || fmt == TPO_FMT_RGBS) {
        float *pl = (float *)out;
        const int nplanes = (fmt == TPO_FMT_GRAYS) ? 1 : 3;
        memset(pl, 0, sizeof(float) * planeSize * nplanes);
        float b[6] = {0, 0, 0, 0, 0, 0};
        if (fmt == TPO_FMT_RGBS) float_rgb_bounds(p, b);
        else float_bounds(p->clamp_mode, b);
        for (int32_t y = 0; y < activeHeight; y++) {
            const int32_t inputLine = p->first_active_frame_line + y;
            const double *inY = cf->y + (size_t)inputLine * cf->width + p->active_start;
            const double *inU = cf->u + (size_t)inputLine * cf->width + p->active_start;
            const double *inV = cf->v + (size_t)inputLine * cf->width + p->active_start;
            const size_t rowOff = (size_t)ow * (tpad + y) + lp;
            for (int32_t x = 0; x < activeWidth; x++) {
                if (fmt == TPO_FMT_RGBS) {
                    const double rY = (inY[x] - yOffset) * eyScale;
                    const double rU = inU[x] * (1.0 / uvRange);
                    const double rV = inV[x] * (1.0 / uvRange);
                    pl[rowOff + x] = fclamp((float)(rY + rFromV * rV), b[0], b[1]);
                    pl[planeSize + rowOff + x] = fclamp((float)(rY + gFromU * rU + gFromV * rV), b[2], b[3]);
                    pl[2 * planeSize + rowOff + x] = fclamp((float)(rY + bFromU * rU), b[4], b[5]);
                    continue;
                }
                pl[rowOff + x] = fclamp((float)((inY[x] - yOffset) * eyScale), b[0], b[1]);
                if (fmt == TPO_FMT_GRAYS) continue;
                pl[planeSize + rowOff + x] = fclamp((float)(inU[x] * ecbScale), b[2], b[3]);
                pl[2 * planeSize + rowOff + x] = fclamp((float)(inV[x] * ecrScale), b[2], b[3]);
            }
        }
        return;
    }
    uint16_t *pl = (uint16_t *)out;
    double b[4];
    int_bounds(p->clamp_mode, b);
    if (fmt == TPO_FMT_RGB48) {
        if (padded) memset(pl, 0, sizeof(uint16_t) * planeSize * 3);
        const double yScale = 65535.0 / yRange;
        const double uvScale = 65535.0 / uvRange;
        for (int32_t y = 0; y < activeHeight; y++) {
            const int32_t inputLine = p->first_active_frame_line + y;
            const double *inY = cf->y + (size_t)inputLine * cf->width + p->active_start;
            const double *inU = cf->u + (size_t)inputLine * cf->width + p->active_start;
            const double *inV = cf->v + (size_t)inputLine * cf->width + p->active_start;
            uint16_t *o = pl + ((size_t)ow * (tpad + y) + lp) * 3;
            for (int32_t x = 0; x < activeWidth; x++) {
                const double rY = dclamp((inY[x] - yOffset) * yScale, 0.0, 65535.0);
                const double rU = inU[x] * uvScale;
                const double rV = inV[x] * uvScale;
                o[3 * x] = (uint16_t)dclamp(rY + (rFromV * rV), 0.0, 65535.0);
                o[3 * x + 1] = (uint16_t)dclamp(rY + (gFromU * rU) + (gFromV * rV), 0.0, 65535.0);
                o[3 * x + 2] = (uint16_t)dclamp(rY + (bFromU * rU), 0.0, 65535.0);
            }
        }
        return;
    }
    const int nplanes = (fmt == TPO_FMT_GRAY16) ? 1 : 3;
    if (padded) {
        for (size_t i = 0; i < planeSize; i++) {
            pl[i] = (uint16_t)(16.0 * 256.0);
            if (nplanes == 3) {
                pl[planeSize + i] = (uint16_t)(128.0 * 256.0);
                pl[2 * planeSize + i] = (uint16_t)(128.0 * 256.0);
            }
        }
    }
    for (int32_t y = 0; y < activeHeight; y++) {
        const int32_t inputLine = p->first_active_frame_line + y;
        const double *inY = cf->y + (size_t)inputLine * cf->width + p->active_start;
        const double *inU = cf->u + (size_t)inputLine * cf->width + p->active_start;
        const double *inV = cf->v + (size_t)inputLine * cf->width + p->active_start;
        const size_t rowOff = (size_t)ow * (tpad + y) + lp;
        for (int32_t x = 0; x < activeWidth; x++) {
            pl[rowOff + x] = (uint16_t)dclamp(h273_round(219.0 * 256.0 * ((inY[x] - yOffset) * eyScale) + 16.0 * 256.0), b[0], b[1]);
            if (nplanes == 1) continue;
            pl[planeSize + rowOff + x] = (uint16_t)dclamp(h273_round(224.0 * 256.0 * (inU[x] * ecbScale) + 128.0 * 256.0), b[2], b[3]);
            pl[2 * planeSize + rowOff + x] = (uint16_t)dclamp(h273_round(224.0 * 256.0 * (inV[x] * ecrScale) + 128.0 * 256.0), b[2], b[3]);
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Dropout concealment, src/dropout/dropout_corrector.cpp:50-530            */
/* ------------------------------------------------------------------------ */

enum { LOC_VISIBLE = 0, LOC_BURST = 1, LOC_UNKNOWN = 2 };

typedef struct do_loc {
    int32_t fieldLine, startx, endx, location;
} do_loc;

typedef struct do_list {
    do_loc *v;
    int32_t n, cap;
} do_list;

static void dl_push(do_list *l, do_loc d)
{
    if (l->n == l->cap) {
        l->cap = l->cap ? 2 * l->cap : 16;
        l->v = (do_loc *)realloc(l->v, sizeof(do_loc) * l->cap);
    }
    l->v[l->n++] = d;
}

/* populateDropoutsVector, dropout_corrector.cpp:160-193 */
static void populate(const tpo_params *p, const tpo_dropout *d, int32_t nd, int32_t field, int32_t overCorrect,
                     do_list *out)
{
    for (int32_t i = 0; i < nd; i++) {
        if (d[i].field != field) continue;
        do_loc l;
        l.startx = d[i].startx;
        l.endx = d[i].endx;
        l.fieldLine = d[i].field_line;
        l.location = LOC_UNKNOWN;
        if (l.fieldLine < 1 || l.fieldLine > p->field_height) continue;
        if (overCorrect) {
            const int32_t dots = 24;
            if (l.startx > dots) l.startx -= dots;
            else l.startx = 0;
            if (l.endx < p->field_width - dots) l.endx += dots;
            else l.endx = p->field_width;
        }
        dl_push(out, l);
    }
}

/* setDropOutLocations, dropout_corrector.cpp:196-245 */
static void set_locations(const tpo_params *p, do_list *d)
{
    int32_t splitCount;
    do {
        const int32_t noOfDropOuts = d->n;
        splitCount = 0;
        for (int32_t index = 0; index < noOfDropOuts; index++) {
            if (d->v[index].startx <= p->burst_end) {
                d->v[index].location = LOC_BURST;
                if (d->v[index].endx > p->burst_end) {
                    do_loc t;
                    t.startx = p->burst_end + 1;
                    t.endx = d->v[index].endx;
                    t.fieldLine = d->v[index].fieldLine;
                    t.location = LOC_BURST;
                    dl_push(d, t);
                    d->v[index].endx = p->burst_end;
                    splitCount++;
                }
            } else if (d->v[index].startx > p->burst_end && d->v[index].startx <= p->active_end) {
                d->v[index].location = LOC_VISIBLE;
                if (d->v[index].endx > p->active_end) {
                    d->v[index].endx = p->active_end;
                    splitCount++;
                }
            }
        }
    } while (splitCount != 0);
}

typedef struct replacement {
    int32_t isSameField, fieldLine, distance, sourceNumber;
    double quality;
} replacement;

static replacement no_replacement(void)
{
    replacement r;
    r.isSameField = 1;
    r.fieldLine = -1;
    r.distance = 0;
    r.sourceNumber = 0;
    r.quality = -1.0;
    return r;
}

/* The captures one frame is concealed from: source 0 is the primary (its
 * broadcast-first and second fields, corrected in place), sources 1.. are
 * the extra captures that hold the frame (DropoutCorrector::correctFrame's
 * multi-source form, dropout_corrector.cpp:50-114). */
#define MAX_SOURCES 9
typedef struct frame_sources {
    int32_t n;
    const uint16_t *first[MAX_SOURCES], *second[MAX_SOURCES];
    do_list fd[MAX_SOURCES], sd[MAX_SOURCES];   /* located dropouts per source */
    double quality[MAX_SOURCES];                /* average VITS bPSNR of the frame's two fields */
} frame_sources;

/* findPotentialReplacementLine, dropout_corrector.cpp:417-466 */
static void find_potential(const tpo_params *p, const do_list *target, int32_t targetIndex, const do_list *source,
                           int32_t isSameField, int32_t sourceOffset, int32_t stepAmount, int32_t sourceNo,
                           double quality, replacement *cands, int32_t *ncand)
{
    const int32_t firstField = (p->first_active_frame_line + 1) / 2; /* core.h firstActiveFieldLine() */
    const int32_t lastField = p->last_active_frame_line / 2;         /* lastActiveFieldLine() */
    int32_t sourceLine = target->v[targetIndex].fieldLine + sourceOffset;
    if ((sourceLine - 1) < firstField || (sourceLine - 1) > lastField) return;
    while ((sourceLine - 1) >= firstField && sourceLine <= lastField) {
        int32_t hasOverlap = 0;
        for (int32_t s = 0; s < source->n; s++) {
            if (source->v[s].fieldLine == sourceLine && (target->v[targetIndex].endx - source->v[s].startx) >= 0 &&
                (source->v[s].endx - target->v[targetIndex].startx) >= 0) {
                sourceLine += stepAmount;
                hasOverlap = 1;
                break;
            }
        }
        if (!hasOverlap) {
            replacement r;
            r.isSameField = isSameField;
            r.fieldLine = sourceLine;
            r.sourceNumber = sourceNo;
            r.quality = quality;
            r.distance = 0;
            cands[(*ncand)++] = r;
            return;
        }
    }
}

/* findReplacementLine, dropout_corrector.cpp:248-414. thisD / otherD hold
 * every source's located dropouts; the target is source 0's entry idx. */
static replacement find_replacement(const tpo_params *p, const do_list *thisD, const do_list *otherD, int32_t nsrc,
                                    const double *quality, int32_t idx, int32_t thisFieldIsFirst,
                                    int32_t matchChromaPhase, int32_t isColourBurst, int32_t intraField)
{
    int32_t stepAmount, otherFieldOffset;
    if (!matchChromaPhase) {
        stepAmount = 1;
        otherFieldOffset = -1;
    } else {
        /* PAL / PAL-M */
        stepAmount = 4;
        otherFieldOffset = thisFieldIsFirst ? -3 : -1;
    }
    replacement cands[4 * MAX_SOURCES];
    int32_t nc = 0;
    for (int32_t s = 0; s < nsrc; s++) {
        find_potential(p, &thisD[0], idx, &thisD[s], 1, 0, -stepAmount, s, quality[s], cands, &nc);
        find_potential(p, &thisD[0], idx, &thisD[s], 1, stepAmount, stepAmount, s, quality[s], cands, &nc);
        if (!isColourBurst && !intraField) {
            find_potential(p, &thisD[0], idx, &otherD[s], 0, otherFieldOffset, -stepAmount, s, quality[s], cands,
                           &nc);
            find_potential(p, &thisD[0], idx, &otherD[s], 0, otherFieldOffset + stepAmount, stepAmount, s,
                           quality[s], cands, &nc);
        }
    }
    replacement rep = no_replacement();
    if (nc > 0) {
        rep.distance = 1000000;
        rep.quality = -1;
        for (int32_t i = 0; i < nc; i++) {
            const int32_t dropoutFrameLine = (2 * thisD[0].v[idx].fieldLine) + (thisFieldIsFirst ? 0 : 1);
            const int32_t sourceFrameLine =
                (2 * cands[i].fieldLine) + (cands[i].isSameField ? (thisFieldIsFirst ? 0 : 1) : (thisFieldIsFirst ? 1 : 0));
            const int32_t distance = abs(dropoutFrameLine - sourceFrameLine);
            if (distance < rep.distance) {
                rep = cands[i];
                rep.distance = distance;
            } else if (distance == rep.distance && cands[i].quality > rep.quality) {
                rep = cands[i];
                rep.distance = distance;
            }
        }
    }
    return rep;
}

/* Filters::palLumaFirFilter and palMLumaFirFilter (= ntscLumaFirFilter),
 * src/dropout/luma_filters.cpp:27-38,60-93, with FIRFilter::apply,
 * src/decoders/filter/firfilter.h:52-99 (zero outside, double accumulation
 * in tap order, truncating store to uint16); the PAL-M taps for system
 * PAL_M (dropout_corrector.cpp:498-506). */
static void pal_luma_fir(uint16_t *data, int32_t n, uint16_t *tmp, int32_t pal_m)
{
    static const double pal[5] = {0.03283437, 0.23959832, 0.45513461, 0.23959832, 0.03283437};
    static const double palm[5] = {0.03275786, 0.23955702, 0.45537024, 0.23955702, 0.03275786};
    const double *coeffs = pal_m ? palm : pal;
    for (int32_t i = 0; i < n; i++) {
        double v = 0;
        for (int32_t j = 0, k = i - 2; j < 5; j++, k++) {
            if (k >= 0 && k < n) v += coeffs[j] * data[k];
        }
        tmp[i] = (uint16_t)v;
    }
    memcpy(data, tmp, sizeof(uint16_t) * (size_t)n);
}

/* correctDropOut, dropout_corrector.cpp:469-530. thisData[0] is the target
 * field; thisData[s] / otherData[s] are source s's fields. */
static void correct_dropout(const tpo_params *p, const do_loc *d, const replacement *rep, const replacement *crep,
                            uint16_t *target, const uint16_t *const *thisData, const uint16_t *const *otherData,
                            uint16_t *lineBuf, uint16_t *tmp)
{
    const int32_t fw = p->field_width;
    if (rep->fieldLine == -1) return;
    const uint16_t *sourceLine =
        (rep->isSameField ? thisData[rep->sourceNumber] : otherData[rep->sourceNumber]) + ((rep->fieldLine - 1) * fw);
    uint16_t *targetLine = target + ((d->fieldLine - 1) * fw);
    if ((crep->fieldLine == -1) || ((d->fieldLine == rep->fieldLine) && (d->fieldLine == crep->fieldLine))) {
        for (int32_t px = d->startx; px < d->endx; px++) targetLine[px] = sourceLine[px];
    } else {
        memcpy(lineBuf, sourceLine, sizeof(uint16_t) * (size_t)fw);
        pal_luma_fir(lineBuf, fw, tmp, p->is_pal_m);
        for (int32_t px = d->startx; px < d->endx; px++) targetLine[px] = lineBuf[px];
        const uint16_t *chromaLine = (crep->isSameField ? thisData[crep->sourceNumber] : otherData[crep->sourceNumber]) +
                                     ((crep->fieldLine - 1) * fw);
        memcpy(lineBuf, chromaLine, sizeof(uint16_t) * (size_t)fw);
        pal_luma_fir(lineBuf, fw, tmp, p->is_pal_m);
        for (int32_t px = d->startx; px < d->endx; px++)
            targetLine[px] = (uint16_t)(targetLine[px] + (chromaLine[px] - lineBuf[px]));
    }
}

/* correctField, dropout_corrector.cpp:117-157 */
static void correct_field(const tpo_params *p, const do_list *thisD, const do_list *otherD, int32_t nsrc,
                          const double *quality, uint16_t *target, const uint16_t *const *thisData,
                          const uint16_t *const *otherData, int32_t thisFieldIsFirst, int32_t intraField,
                          tpo_stats *stats)
{
    uint16_t *lineBuf = (uint16_t *)malloc(sizeof(uint16_t) * 2 * (size_t)p->field_width);
    uint16_t *tmp = lineBuf + p->field_width;
    for (int32_t i = 0; i < thisD[0].n; i++) {
        replacement rep = no_replacement(), crep = no_replacement();
        if (thisD[0].v[i].location == LOC_BURST)
            rep = find_replacement(p, thisD, otherD, nsrc, quality, i, thisFieldIsFirst, 1, 1, intraField);
        if (thisD[0].v[i].location == LOC_VISIBLE) {
            rep = find_replacement(p, thisD, otherD, nsrc, quality, i, thisFieldIsFirst, 0, 0, intraField);
            crep = find_replacement(p, thisD, otherD, nsrc, quality, i, thisFieldIsFirst, 1, 0, intraField);
        }
        if (stats) {
            if (rep.fieldLine == -1) {
                stats->failed++;
            } else {
                stats->corrected++;
                stats->total_distance += rep.distance;
            }
        }
        correct_dropout(p, &thisD[0].v[i], &rep, &crep, target, thisData, otherData, lineBuf, tmp);
    }
    free(lineBuf);
}

static int32_t frame_dropouts(const tpo_params *p, const tpo_dropout *d, int32_t nd, int32_t frame,
                              tpo_dropout **out);
static void shift_field(const tpo_params *p, const uint16_t *src, uint16_t *dst);

/* DropoutCorrector::correctFrame, dropout_corrector.cpp:40-114, with the
 * extra sources decodeSourceFrame passes (c_api_decoder.cpp:245-297). The
 * primary's two fields are taken in broadcast order: `first` is the field
 * whose metadata says isFirstField (capture field index fi_first), `second`
 * the other one. d holds the frame's dropouts as loaded (shifted for a
 * subcarrier-locked second field). An extra source contributes the frame
 * its frame_map gives for primary frame `frame`, its slot-0 field as
 * "first" and slot-1 field (shifted when subcarrier-locked) as "second",
 * the way decodeSourceFrame reads getFirstFieldNumber / getSecondFieldNumber;
 * extras without the frame are left out. */
static void correct_frame(const tpo_params *p, const tpo_dropout *d, int32_t nd, int32_t fi_first,
                          int32_t fi_second, uint16_t *first, uint16_t *second, int32_t overCorrect,
                          int32_t intraField, tpo_stats *stats, const tpo_sources *src, int32_t frame)
{
    /* "Skip if no dropouts in primary fields" tests the metadata lists, which
     * also hold entries populate() drops for being off the field. */
    int32_t any = 0;
    for (int32_t i = 0; i < nd; i++)
        if (d[i].field == fi_first || d[i].field == fi_second) any = 1;
    if (!any) return;
    const size_t fl = (size_t)p->field_width * p->field_height;
    frame_sources fs;
    memset(&fs, 0, sizeof(fs));
    uint16_t *shifted[MAX_SOURCES] = {0};
    fs.n = 1;
    fs.first[0] = first;
    fs.second[0] = second;
    fs.quality[0] = (src && src->bpsnr) ? (src->bpsnr[fi_first] + src->bpsnr[fi_second]) / 2.0 : 0.0;
    populate(p, d, nd, fi_first, overCorrect, &fs.fd[0]);
    populate(p, d, nd, fi_second, overCorrect, &fs.sd[0]);
    for (int32_t e = 0; src && e < src->nextras && fs.n < MAX_SOURCES; e++) {
        const tpo_extra *x = &src->extras[e];
        const int32_t k = x->frame_map ? (frame < x->nframe_map ? x->frame_map[frame] : -1) : frame;
        if (k < 0 || k >= x->nfields / 2) continue;
        const int32_t s = fs.n++;
        fs.first[s] = x->fields + fl * (size_t)(2 * k);
        fs.second[s] = x->fields + fl * (size_t)(2 * k + 1);
        if (p->sc_locked) {
            shifted[s] = (uint16_t *)malloc(sizeof(uint16_t) * fl);
            shift_field(p, fs.second[s], shifted[s]);
            fs.second[s] = shifted[s];
        }
        fs.quality[s] = x->bpsnr ? (x->bpsnr[2 * k] + x->bpsnr[2 * k + 1]) / 2.0 : 0.0;
        tpo_dropout *xd = NULL;
        const int32_t nxd = x->dropouts ? frame_dropouts(p, x->dropouts, x->ndropouts, k, &xd) : 0;
        populate(p, xd, nxd, 2 * k, overCorrect, &fs.fd[s]);
        populate(p, xd, nxd, 2 * k + 1, overCorrect, &fs.sd[s]);
        free(xd);
    }
    for (int32_t s = 0; s < fs.n; s++) {
        if (fs.fd[s].n) set_locations(p, &fs.fd[s]);
        if (fs.sd[s].n) set_locations(p, &fs.sd[s]);
    }
    correct_field(p, fs.fd, fs.sd, fs.n, fs.quality, first, fs.first, fs.second, 1, intraField, stats);
    correct_field(p, fs.sd, fs.fd, fs.n, fs.quality, second, fs.second, fs.first, 0, intraField, stats);
    for (int32_t s = 0; s < fs.n; s++) {
        free(fs.fd[s].v);
        free(fs.sd[s].v);
        free(shifted[s]);
    }
}

/* The dropouts of frame `frame` as SourceField::loadFields leaves them: a
 * subcarrier-locked slot-1 field's dropouts move 2 samples left and vanish
 * when they end at or before sample 0 (source_field.cpp:51-66). Returns the
 * count; *out is malloc'd (free it). */
static int32_t frame_dropouts(const tpo_params *p, const tpo_dropout *d, int32_t nd, int32_t frame,
                              tpo_dropout **out)
{
    *out = NULL;
    int32_t n = 0;
    for (int32_t i = 0; i < nd; i++)
        if (d[i].field == 2 * frame || d[i].field == 2 * frame + 1) n++;
    if (n == 0) return 0;
    tpo_dropout *v = (tpo_dropout *)malloc(sizeof(tpo_dropout) * (size_t)n);
    int32_t k = 0;
    for (int32_t i = 0; i < nd; i++) {
        if (d[i].field != 2 * frame && d[i].field != 2 * frame + 1) continue;
        tpo_dropout x = d[i];
        if (p->sc_locked && x.field == 2 * frame + 1) {
            const int32_t endx = x.endx - 2;
            if (endx <= 0) continue;
            x.startx = imax(x.startx - 2, 0);
            x.endx = endx;
        }
        v[k++] = x;
    }
    *out = v;
    return k;
}

/* shiftSecondField's samples: drop the first 2, append 2 black (source_field.cpp:51-57). */
static void shift_field(const tpo_params *p, const uint16_t *src, uint16_t *dst)
{
    const size_t fl = (size_t)p->field_width * p->field_height;
    memcpy(dst, src + 2, sizeof(uint16_t) * (fl - 2));
    dst[fl - 2] = (uint16_t)p->black;
    dst[fl - 1] = (uint16_t)p->black;
}

/* Correct frame f's fields c0 (slot 0) and c1 (slot 1) in place; stats of the correction. */
static void correct_slots(const tpo_params *p, const tpo_dropout *fd, int32_t nfd, int32_t f, uint16_t *c0,
                          uint16_t *c1, int32_t overcorrect, int32_t intra, tpo_stats *st, const tpo_sources *src)
{
    if (p->first_field_offset == 0)
        correct_frame(p, fd, nfd, 2 * f, 2 * f + 1, c0, c1, overcorrect, intra, st, src, f);
    else
        correct_frame(p, fd, nfd, 2 * f + 1, 2 * f, c1, c0, overcorrect, intra, st, src, f);
}

/* ------------------------------------------------------------------------ */
/* Frame decode                                                             */
/* ------------------------------------------------------------------------ */

typedef struct decoder {
    tpo_params p;
    tp_ctx tp;
    pal_ctx pal;
    demod_scratch *scratch;
    component_frame cf;
    uint16_t *black;       /* one black field */
    uint16_t *corrected;   /* window frames' corrected / shifted copies, 2 fields per frame */
} decoder;

static int decoder_init(decoder *d, const tpo_params *p)
{
    memset(d, 0, sizeof(*d));
    d->p = *p;
    if (tp_init(&d->tp, p) != 0) return -1;
    pal_build(&d->pal, p);
    d->scratch = (demod_scratch *)calloc(1, sizeof(demod_scratch));
    d->cf.width = p->field_width;
    d->cf.height = 2 * p->field_height - 1;
    const size_t n = (size_t)d->cf.width * d->cf.height;
    d->cf.y = (double *)malloc(sizeof(double) * n * 3);
    d->cf.u = d->cf.y + n;
    d->cf.v = d->cf.u + n;
    const size_t fl = (size_t)p->field_width * p->field_height;
    d->black = (uint16_t *)malloc(sizeof(uint16_t) * fl);
    for (size_t i = 0; i < fl; i++) d->black[i] = (uint16_t)p->black;
    d->corrected = (uint16_t *)malloc(sizeof(uint16_t) * fl * 2 * 8);
    return (d->scratch && d->cf.y && d->black && d->corrected) ? 0 : -1;
}

static void decoder_free(decoder *d)
{
    tp_free(&d->tp);
    free(d->scratch);
    free(d->cf.y);
    free(d->black);
    free(d->corrected);
}

static int32_t look_behind(const tpo_params *p) { return p->kind == 3 ? (4 + 1) / 2 : 0; } /* transform_pal_3d.cpp:111-115; 0 for 2D and PALcolour */
static int32_t look_ahead(const tpo_params *p) { return p->kind == 3 ? (8 - 1 + 1) / 2 : 0; } /* :117-121 */

/* Window of frames [frame-lb, frame+1+la) with black padding outside the
 * capture (source_field.cpp:88-170) and dropout concealment of every
 * non-padding window frame that has dropouts (c_api_decoder.cpp:300-321). */
static int32_t load_window(decoder *d, const uint16_t *fields, int32_t nfields, const tpo_dropout *drops,
                           int32_t nd, int32_t overcorrect, int32_t intra, int32_t frame, int32_t lb, int32_t la,
                           src_field *win, tpo_stats *stats, const tpo_sources *src)
{
    const tpo_params *p = &d->p;
    const size_t fl = (size_t)p->field_width * p->field_height;
    const int32_t numFrames = nfields / 2;
    const int32_t n = 2 * (lb + 1 + la);
    for (int32_t i = 0; i < n; i += 2) {
        const int32_t f = frame - lb + i / 2;
        win[i].offset = p->first_field_offset;
        win[i + 1].offset = 1 - p->first_field_offset;
        if (f < 0 || f >= numFrames) {
            win[i].data = d->black;
            win[i + 1].data = d->black;
            continue;
        }
        win[i].data = fields + fl * (size_t)(2 * f);
        win[i + 1].data = fields + fl * (size_t)(2 * f + 1);
        uint16_t *c0 = d->corrected + fl * (size_t)i;
        uint16_t *c1 = c0 + fl;
        if (p->sc_locked) {   /* SourceField::shiftSecondField on slot 1 */
            shift_field(p, win[i + 1].data, c1);
            win[i + 1].data = c1;
        }
        tpo_dropout *fd = NULL;
        const int32_t nfd = drops ? frame_dropouts(p, drops, nd, f, &fd) : 0;
        if (nfd > 0) {
            if (win[i].data != c0) memcpy(c0, win[i].data, sizeof(uint16_t) * fl);
            if (win[i + 1].data != c1) memcpy(c1, win[i + 1].data, sizeof(uint16_t) * fl);
            tpo_stats st = {0, 0, 0};
            correct_slots(p, fd, nfd, f, c0, c1, overcorrect, intra, &st, src);
            if (f == frame && stats) {
                stats->corrected += st.corrected;
                stats->failed += st.failed;
                stats->total_distance += st.total_distance;
            }
            win[i].data = c0;
            win[i + 1].data = c1;
        }
        free(fd);
    }
    return 2 * lb; /* startIndex */
}

static int decode_one(decoder *d, const uint16_t *fields, int32_t nfields, const tpo_dropout *drops, int32_t nd,
                      int32_t overcorrect, int32_t intra, int32_t frame, void *out, tpo_stats *stats,
                      const tpo_sources *src)
{
    const tpo_params *p = &d->p;
    const size_t fl = (size_t)p->field_width * p->field_height;
    src_field win[16];
    const int32_t lb = look_behind(p), la = look_ahead(p);
    const int32_t startIndex =
        load_window(d, fields, nfields, drops, nd, overcorrect, intra, frame, lb, la, win, stats, src);
    double *chroma[2];
    for (int j = 0; j < 2; j++) {
        if (d->tp.nchroma <= j) {
            d->tp.chroma[j] = (double *)malloc(sizeof(double) * fl);
            d->tp.nchroma = j + 1;
        }
        chroma[j] = d->tp.chroma[j];
        memset(chroma[j], 0, sizeof(double) * fl);
    }
    if (p->kind == 2) {
        filter_field_2d(&d->tp, p, &win[startIndex], chroma[0]);
        filter_field_2d(&d->tp, p, &win[startIndex + 1], chroma[1]);
    } else if (p->kind == 3) {
        filter_fields_3d(&d->tp, p, win, startIndex, startIndex + 2, chroma);
    }
    const size_t n = (size_t)d->cf.width * d->cf.height;
    memset(d->cf.y, 0, sizeof(double) * n * 3);
    decode_field(&d->pal, p, &win[startIndex], chroma[0], &d->cf, d->scratch);
    decode_field(&d->pal, p, &win[startIndex + 1], chroma[1], &d->cf, d->scratch);
    write_output(p, &d->cf, out);
    return 0;
}

typedef struct job {
    const tpo_params *p;
    const uint16_t *fields;
    int32_t nfields;
    const tpo_dropout *drops;
    int32_t nd, overcorrect, intra, first, count;
    uint8_t *out;
    size_t frameBytes;
    atomic_int next;
    atomic_int err;
    tpo_stats *stats;
    pthread_mutex_t statsMu;
    const tpo_sources *src;
} job;

static void *worker(void *arg)
{
    job *j = (job *)arg;
    decoder d;
    if (decoder_init(&d, j->p) != 0) {
        atomic_store(&j->err, 1);
        decoder_free(&d);
        return NULL;
    }
    for (;;) {
        const int32_t i = atomic_fetch_add(&j->next, 1);
        if (i >= j->count) break;
        tpo_stats st = {0, 0, 0};
        decode_one(&d, j->fields, j->nfields, j->drops, j->nd, j->overcorrect, j->intra, j->first + i,
                   j->out + (size_t)i * j->frameBytes, &st, j->src);
        if (j->stats) {
            pthread_mutex_lock(&j->statsMu);
            j->stats->corrected += st.corrected;
            j->stats->failed += st.failed;
            j->stats->total_distance += st.total_distance;
            pthread_mutex_unlock(&j->statsMu);
        }
    }
    decoder_free(&d);
    return NULL;
}

int tpo_decode_frames(const tpo_params *p, const uint16_t *fields, int32_t nfields, const tpo_dropout *dropouts,
                      int32_t ndropouts, int32_t overcorrect, int32_t intra_field, int32_t first, int32_t count,
                      void *out, int32_t nthreads, tpo_stats *stats)
{
    return tpo_decode_frames_ms(p, fields, nfields, dropouts, ndropouts, NULL, overcorrect, intra_field, first, count,
                                out, nthreads, stats);
}

int tpo_decode_frames_ms(const tpo_params *p, const uint16_t *fields, int32_t nfields, const tpo_dropout *dropouts,
                         int32_t ndropouts, const tpo_sources *sources, int32_t overcorrect, int32_t intra_field,
                         int32_t first, int32_t count, void *out, int32_t nthreads, tpo_stats *stats)
{
    if (sources && (sources->nextras < 0 || sources->nextras > MAX_SOURCES - 1)) return -1;
    if (!p || !fields || !out || count < 0 || (p->kind != 1 && p->kind != 2 && p->kind != 3)) return -1;
    if (p->output_format < TPO_FMT_P16 || p->output_format > TPO_FMT_GRAYS) return -1;
    if (p->thresholds && p->n_thresholds != (p->kind == 2 ? 80 : 768)) return -1;
    job j;
    j.p = p;
    j.fields = fields;
    j.nfields = nfields;
    j.drops = (ndropouts > 0) ? dropouts : NULL;
    j.nd = ndropouts;
    j.overcorrect = overcorrect;
    j.intra = intra_field;
    j.first = first;
    j.count = count;
    j.out = (uint8_t *)out;
    j.frameBytes = tpo_frame_bytes(p);
    atomic_init(&j.next, 0);
    atomic_init(&j.err, 0);
    j.stats = stats;
    j.src = sources;
    if (stats) memset(stats, 0, sizeof(*stats));
    pthread_mutex_init(&j.statsMu, NULL);
    if (nthreads < 1) nthreads = 1;
    if (nthreads > count) nthreads = count > 0 ? count : 1;
    pthread_t th[256];
    if (nthreads > 256) nthreads = 256;
    if (nthreads == 1) {
        worker(&j);
    } else {
        for (int32_t i = 0; i < nthreads; i++) pthread_create(&th[i], NULL, worker, &j);
        for (int32_t i = 0; i < nthreads; i++) pthread_join(th[i], NULL);
    }
    pthread_mutex_destroy(&j.statsMu);
    return atomic_load(&j.err) ? -1 : 0;
}

int tpo_transform_chroma(const tpo_params *p, const uint16_t *fields, int32_t nfields, int32_t first, int32_t count,
                         double *out)
{
    decoder d;
    if (decoder_init(&d, p) != 0) {
        decoder_free(&d);
        return -1;
    }
    const size_t fl = (size_t)p->field_width * p->field_height;
    for (int32_t k = 0; k < count; k++) {
        src_field win[16];
        const int32_t lb = look_behind(p), la = look_ahead(p);
        const int32_t startIndex = load_window(&d, fields, nfields, NULL, 0, 0, 0, first + k, lb, la, win, NULL, NULL);
        double *chroma[2] = {out + fl * (size_t)(2 * k), out + fl * (size_t)(2 * k + 1)};
        memset(chroma[0], 0, sizeof(double) * fl * 2);
        if (p->kind == 2) {
            filter_field_2d(&d.tp, p, &win[startIndex], chroma[0]);
            filter_field_2d(&d.tp, p, &win[startIndex + 1], chroma[1]);
        } else {
            filter_fields_3d(&d.tp, p, win, startIndex, startIndex + 2, chroma);
        }
    }
    decoder_free(&d);
    return 0;
}

int tpo_dropout_correct_frame(const tpo_params *p, const uint16_t *fields, int32_t nfields,
                              const tpo_dropout *dropouts, int32_t ndropouts, int32_t overcorrect,
                              int32_t intra_field, int32_t frame, uint16_t *out, tpo_stats *stats)
{
    return tpo_dropout_correct_frame_ms(p, fields, nfields, dropouts, ndropouts, NULL, overcorrect, intra_field,
                                        frame, out, stats);
}

int tpo_dropout_correct_frame_ms(const tpo_params *p, const uint16_t *fields, int32_t nfields,
                                 const tpo_dropout *dropouts, int32_t ndropouts, const tpo_sources *sources,
                                 int32_t overcorrect, int32_t intra_field, int32_t frame, uint16_t *out,
                                 tpo_stats *stats)
{
    if (sources && (sources->nextras < 0 || sources->nextras > MAX_SOURCES - 1)) return -1;
    const size_t fl = (size_t)p->field_width * p->field_height;
    if (frame < 0 || 2 * frame + 1 >= nfields) return -1;
    memcpy(out, fields + fl * (size_t)(2 * frame), sizeof(uint16_t) * fl);
    if (p->sc_locked) shift_field(p, fields + fl * (size_t)(2 * frame + 1), out + fl);
    else memcpy(out + fl, fields + fl * (size_t)(2 * frame + 1), sizeof(uint16_t) * fl);
    tpo_stats st = {0, 0, 0};
    tpo_dropout *fd = NULL;
    const int32_t nfd = frame_dropouts(p, dropouts, ndropouts, frame, &fd);
    if (nfd > 0) correct_slots(p, fd, nfd, frame, out, out + fl, overcorrect, intra_field, &st, sources);
    free(fd);
    if (stats) *stats = st;
    return 0;
}

static int span_cmp(const void *a, const void *b)
{
    const tpo_span *x = (const tpo_span *)a, *y = (const tpo_span *)b;
    if (x->y != y->y) return x->y < y->y ? -1 : 1;
    if (x->x_start != y->x_start) return x->x_start < y->x_start ? -1 : 1;
    if (x->x_end != y->x_end) return x->x_end < y->x_end ? -1 : 1;
    return 0;
}

/* appendFieldSpans / collectSpans, src/abi/c_api_dropout_detect.cpp:92-174 */
int32_t tpo_dropout_spans(const tpo_params *p, const tpo_dropout *d, int32_t nd, int32_t frame, int32_t mode,
                          tpo_span *out, int32_t cap)
{
    int32_t ow, oh, lp, tpad;
    tpo_output_geometry(p, &ow, &oh, &lp, &tpad);
    const int32_t avs = p->active_start;
    const int32_t ave = p->active_end;
    int32_t n = 0;
    tpo_dropout *fd = NULL;
    const int32_t nfd = frame_dropouts(p, d, nd, frame, &fd);
    for (int32_t j = 0; j < 2; j++) {
        const int32_t field = 2 * frame + j;
        const int32_t offset = j ^ p->first_field_offset;   /* SourceField::getOffset */
        for (int32_t i = 0; i < nfd; i++) {
            if (fd[i].field != field) continue;
            const int32_t frameRow = (2 * (fd[i].field_line - 1)) + offset;
            const int32_t y = tpad + frameRow - p->first_active_frame_line;
            if (y < 0 || y >= oh) continue;
            int32_t x0 = fd[i].startx, x1 = fd[i].endx;
            if (mode == 1) {
                const int32_t dots = 24;
                x0 = (x0 > dots) ? x0 - dots : 0;
                x1 = (x1 < p->field_width - dots) ? x1 + dots : p->field_width;
            }
            if (x0 < avs) x0 = avs;
            if (x1 > ave) x1 = ave;
            if (x1 <= x0) continue;
            if (n < cap) {
                out[n].y = y;
                out[n].x_start = x0 - avs + lp;
                out[n].x_end = x1 - avs + lp;
                out[n].origin = 0;
            }
            n++;
        }
    }
    free(fd);
    qsort(out, (size_t)(n < cap ? n : cap), sizeof(tpo_span), span_cmp);
    return n;
}
