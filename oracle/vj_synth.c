/*
 * vj_synth.c - the seeded synthetic inputs, restated in plain C for the
 * oracle (test infrastructure, part of liboracle.so).
 *
 * The reference trains and detects on Kaggle faces, COCO negatives and a demo
 * image, none of which exist offline; the package's generators
 * (cs677s26_gb300/csrc/synth.cpp) stand in for them.  This file computes the
 * same bytes independently, so the CPU legs of the benchmark and the fixture
 * scripts can build their inputs without loading the product library, and
 * tests/test_synth_oracle.py checks that both give identical bytes.
 *
 * Everything is integer arithmetic or single IEEE double/float operations
 * (+ - * / sqrt; no libm transcendental), compiled with -ffp-contract=off,
 * so the bytes are the same on every machine.
 *
 * Generators: xoshiro256** seeded through splitmix64; pink (1/f) texture as
 * equal-amplitude octaves of bilinear value noise on a hashed lattice, scaled
 * to mean 110 / std 45; face patterns (gradient ellipse around 140, eyes -50,
 * mouth band -35, noise sigma 12) on texture; scenes of texture with faces
 * pasted at log-uniform sizes; a cascade with stage sizes 1, 10, 25, 25, 50,
 * then the rest spread evenly, thresholds at random quantiles and stage
 * thresholds at about half rejection of texture windows.
 */
#include "vj_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define WIN 24
#define IIW 25
#define IIAREA (IIW * IIW)

static uint64_t sm_mix(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

typedef struct {
    uint64_t s[4];
} xo_rng;

static xo_rng xo_seed(uint64_t seed) {
    xo_rng r;
    uint64_t z = seed;
    for (int k = 0; k < 4; ++k) {
        z += 0x9E3779B97F4A7C15ull;
        r.s[k] = sm_mix(z);
    }
    return r;
}

static uint64_t rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

static uint64_t xo_next(xo_rng* r) {
    uint64_t* s = r->s;
    const uint64_t out = rotl64(s[1] * 5, 7) * 9;
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl64(s[3], 45);
    return out;
}

/* uniform integer in [lo, hi] */
static int xo_range(xo_rng* r, int lo, int hi) {
    const uint64_t span = (uint64_t)(hi - lo) + 1;
    return lo + (int)(xo_next(r) % span);
}

/* Irwin-Hall sum of the four 16-bit fields of one draw (mean 131070, std
 * 37837.2), rescaled to standard deviation sigma, truncated toward zero */
static int xo_gauss(xo_rng* r, int sigma) {
    const uint64_t v = xo_next(r);
    const int64_t s = (int64_t)(v & 0xFFFF) + (int64_t)((v >> 16) & 0xFFFF) + (int64_t)((v >> 32) & 0xFFFF) +
                      (int64_t)(v >> 48);
    return (int)(((s * 2 - 262140) * sigma) / 75674);
}

static int64_t fdiv64(int64_t a, int64_t b) {
    int64_t q = a / b;
    if ((a % b != 0) && ((a < 0) != (b < 0))) --q;
    return q;
}

static uint8_t sat_u8(int64_t v) { return (uint8_t)(v < 0 ? 0 : (v > 255 ? 255 : v)); }

/* r^(k/1024) from ten correctly rounded square roots */
static double pow_k1024(double r, int k) {
    double roots[10];
    double v = r;
    for (int j = 0; j < 10; ++j) {
        v = sqrt(v);
        roots[j] = v;
    }
    double out = 1.0;
    for (int j = 0; j < 10; ++j)
        if (k & (512 >> j)) out *= roots[j];
    if (k >= 1024) out *= r;
    return out;
}

static int log_uniform_int(xo_rng* r, int lo, int hi) {
    const int k = xo_range(r, 0, 1024);
    const double v = (double)lo * pow_k1024((double)hi / lo, k);
    int out = (int)floor(v + 0.5);
    if (out < lo) out = lo;
    if (out > hi) out = hi;
    return out;
}

/* Pink texture of w x h into out (row stride `stride`). */
static void pink(uint64_t seed, int w, int h, uint8_t* out, int stride) {
    const int64_t npx = (int64_t)w * h;
    int32_t* acc = (int32_t*)calloc((size_t)npx, sizeof(int32_t));
    int maxCell = w > h ? w : h;
    if (maxCell < 2) maxCell = 2;
    if (maxCell > 256) maxCell = 256;
    xo_rng orng = xo_seed(seed ^ 0x5eed7e47u);
    int32_t* grid = NULL;
    size_t gridCap = 0;
    for (int cell = 2, oct = 0; cell <= maxCell; cell *= 2, ++oct) {
        const int offx = xo_range(&orng, 0, cell - 1);
        const int offy = xo_range(&orng, 0, cell - 1);
        const uint64_t oseed = sm_mix(seed * 0x100000001B3ull + (uint64_t)oct);
        const int gw = (w - 1 + offx) / cell + 2;
        const int gh = (h - 1 + offy) / cell + 2;
        if ((size_t)gw * gh > gridCap) {
            gridCap = (size_t)gw * gh;
            grid = (int32_t*)realloc(grid, gridCap * sizeof(int32_t));
        }
        for (int gy = 0; gy < gh; ++gy)
            for (int gx = 0; gx < gw; ++gx) {
                const uint64_t hv = sm_mix(oseed ^ ((uint64_t)gx * 0xC2B2AE3D27D4EB4Full) ^
                                           ((uint64_t)gy * 0x165667B19E3779F9ull));
                grid[(size_t)gy * gw + gx] = (int32_t)(hv & 0xFFFF) - 32768;
            }
        const int64_t c2 = (int64_t)cell * cell;
        for (int y = 0; y < h; ++y) {
            const int iy = (y + offy) / cell;
            const int64_t fy = (y + offy) - (int64_t)iy * cell;
            const int32_t* g0 = grid + (size_t)iy * gw;
            const int32_t* g1 = g0 + gw;
            for (int x = 0; x < w; ++x) {
                const int ix = (x + offx) / cell;
                const int64_t fx = (x + offx) - (int64_t)ix * cell;
                const int64_t top = (int64_t)g0[ix] * (cell - fx) + (int64_t)g0[ix + 1] * fx;
                const int64_t bot = (int64_t)g1[ix] * (cell - fx) + (int64_t)g1[ix + 1] * fx;
                acc[(size_t)y * w + x] += (int32_t)fdiv64(top * (cell - fy) + bot * fy, c2);
            }
        }
    }
    free(grid);
    double sum = 0.0;
    for (int64_t i = 0; i < npx; ++i) sum += (double)acc[i];
    const double mean = sum / (double)npx;
    double ss = 0.0;
    for (int64_t i = 0; i < npx; ++i) {
        const double d = (double)acc[i] - mean;
        ss += d * d;
    }
    double sd = sqrt(ss / (double)npx);
    if (!(sd > 0.0)) sd = 1.0;
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
            const double d = (double)acc[(size_t)y * w + x] - mean;
            const double v = 110.0 + 45.0 * (d / sd);
            out[(size_t)y * stride + x] = sat_u8((int64_t)floor(v + 0.5));
        }
    free(acc);
}

/* One 24x24 face pattern; geometry in quarter pixels. */
static void face24(xo_rng* r, uint8_t* p) {
    pink(xo_next(r), WIN, WIN, p, WIN);
    const int cx = 48 + xo_range(r, -4, 4);
    const int cy = 48 + xo_range(r, -4, 4);
    const int a = 36 + xo_range(r, -3, 3);
    const int b = 44 + xo_range(r, -3, 3);
    const int grad = xo_range(r, -15, 15);
    const int eyeDx = 16 + xo_range(r, -2, 2);
    const int eyeDy = 12 + xo_range(r, -2, 2);
    const int ea = 10, eb = 6;
    const int64_t a2 = (int64_t)a * a, b2 = (int64_t)b * b;
    for (int y = 0; y < WIN; ++y)
        for (int x = 0; x < WIN; ++x) {
            const int dx = 4 * x + 2 - cx, dy = 4 * y + 2 - cy;
            int v = p[y * WIN + x];
            if ((int64_t)dx * dx * b2 + (int64_t)dy * dy * a2 <= a2 * b2) {
                v = 140 + (grad * dy) / b;
                for (int side = -1; side <= 1; side += 2) {
                    const int ex = dx - side * eyeDx, ey = dy + eyeDy;
                    if (ex * ex * eb * eb + ey * ey * ea * ea <= ea * ea * eb * eb) v -= 50;
                }
                if (dx >= -16 && dx <= 16 && dy >= 16 && dy < 24) v -= 35;
            }
            v += xo_gauss(r, 12);
            p[y * WIN + x] = sat_u8(v);
        }
}

/* Bilinear 16.16 fixed-point resize of a 24x24 pattern to s x s at (x0, y0). */
static void paste24(const uint8_t* src, int s, uint8_t* dst, int stride, int x0, int y0) {
    for (int y = 0; y < s; ++y) {
        const int64_t fy = ((2LL * y + 1) * WIN * 65536) / (2LL * s) - 32768;
        int64_t sy = fdiv64(fy, 65536), ay = fy - fdiv64(fy, 65536) * 65536;
        if (sy < 0) {
            sy = 0;
            ay = 0;
        }
        if (sy >= WIN - 1) {
            sy = WIN - 1;
            ay = 0;
        }
        const int64_t sy1 = sy + 1 < WIN - 1 ? sy + 1 : WIN - 1;
        for (int x = 0; x < s; ++x) {
            const int64_t fx = ((2LL * x + 1) * WIN * 65536) / (2LL * s) - 32768;
            int64_t sx = fdiv64(fx, 65536), ax = fx - fdiv64(fx, 65536) * 65536;
            if (sx < 0) {
                sx = 0;
                ax = 0;
            }
            if (sx >= WIN - 1) {
                sx = WIN - 1;
                ax = 0;
            }
            const int64_t sx1 = sx + 1 < WIN - 1 ? sx + 1 : WIN - 1;
            const int64_t top = (int64_t)src[sy * WIN + sx] * (65536 - ax) + (int64_t)src[sy * WIN + sx1] * ax;
            const int64_t bot = (int64_t)src[sy1 * WIN + sx] * (65536 - ax) + (int64_t)src[sy1 * WIN + sx1] * ax;
            dst[(size_t)(y0 + y) * stride + (x0 + x)] = sat_u8((top * (65536 - ay) + bot * ay + (1LL << 31)) >> 32);
        }
    }
}

void vjo_synth_patches(uint64_t seed, int nPos, int nNeg, uint8_t* out) {
    for (int i = 0; i < nPos; ++i) {
        xo_rng r = xo_seed(sm_mix(seed * 0x9E3779B97F4A7C15ull + 0x1000000ull + (uint64_t)i));
        face24(&r, out + (size_t)i * WIN * WIN);
    }
    for (int i = 0; i < nNeg; ++i)
        pink(sm_mix(seed * 0x9E3779B97F4A7C15ull + 0x2000000000ull + (uint64_t)i), WIN, WIN,
             out + (size_t)(nPos + i) * WIN * WIN, WIN);
}

int vjo_synth_scene(uint64_t seed, int w, int h, int nPaste, int minSize, int maxSize, uint8_t* out) {
    if (!out || w < WIN || h < WIN || nPaste < 0 || minSize < 1 || maxSize < minSize) return -1;
    pink(sm_mix(seed ^ 0xA5A5A5A5ull), w, h, out, w);
    xo_rng r = xo_seed(sm_mix(seed + 0x3C3C3C3Cull));
    uint8_t pat[WIN * WIN];
    int smax = maxSize < w ? maxSize : w;
    if (h < smax) smax = h;
    const int smin = minSize < smax ? minSize : smax;
    for (int k = 0; k < nPaste; ++k) {
        const int s = log_uniform_int(&r, smin, smax);
        const int x0 = xo_range(&r, 0, w - s);
        const int y0 = xo_range(&r, 0, h - s);
        xo_rng fr = xo_seed(xo_next(&r));
        face24(&fr, pat);
        paste24(pat, s, out, w, x0, y0);
    }
    return 0;
}

/* A window's integral and its detection-style normalisation (0 = gated). */
typedef struct {
    int32_t sum[IIAREA];
    float inv;
} cal_window;

static void cal_ii(const uint8_t* p, cal_window* c) {
    int64_t sq[IIAREA];
    memset(c->sum, 0, sizeof(c->sum));
    memset(sq, 0, sizeof(sq));
    for (int y = 1; y <= WIN; ++y) {
        int32_t rs = 0;
        int64_t rq = 0;
        for (int x = 1; x <= WIN; ++x) {
            const int v = p[(y - 1) * WIN + (x - 1)];
            rs += v;
            rq += v * v;
            c->sum[y * IIW + x] = c->sum[(y - 1) * IIW + x] + rs;
            sq[y * IIW + x] = sq[(y - 1) * IIW + x] + rq;
        }
    }
    const int q0 = IIW + 1, q1 = IIW + 23, q2 = 23 * IIW + 1, q3 = 23 * IIW + 23;
    const double s = (double)(c->sum[q0] - c->sum[q1] - c->sum[q2] + c->sum[q3]);
    const double ss = (double)(sq[q0] - sq[q1] - sq[q2] + sq[q3]);
    const double nf2 = 484.0 * ss - s * s;
    c->inv = 0.0f;
    if (nf2 > 0.0) {
        const float inv = (float)(1.0 / sqrt(nf2));
        if (484.0 * (double)inv < 0.1) c->inv = inv;
    }
}

static float cal_rect(const vjo_rect* q, const cal_window* c) {
    return ((float)c->sum[q->p0] - (float)c->sum[q->p1] - (float)c->sum[q->p2] + (float)c->sum[q->p3]) * q->w;
}

static float cal_response(const vjo_feature* f, const cal_window* c) {
    float raw = cal_rect(&f->r0, c) + cal_rect(&f->r1, c);
    if (f->rectCount == 3) raw += cal_rect(&f->r2, c);
    return raw * c->inv;
}

static int cmp_float(const void* a, const void* b) {
    const float x = *(const float*)a, y = *(const float*)b;
    return x < y ? -1 : (x > y ? 1 : 0);
}

int vjo_synth_cascade(uint64_t seed, int stageCount, int totalStumps, vjo_stump* stumps, vjo_stage* stages) {
    static const int head[5] = {1, 10, 25, 25, 50};
    if (!stumps || !stages || stageCount < 1 || totalStumps < stageCount) return -1;
    int* sizes = (int*)malloc(sizeof(int) * (size_t)stageCount);
    int used = 0, ns = 0;
    for (int i = 0; i < stageCount && i < 5; ++i) {
        int take = totalStumps - used - (stageCount - i - 1);
        if (head[i] < take) take = head[i];
        sizes[ns] = take > 1 ? take : 1;
        used += sizes[ns++];
    }
    const int rest = stageCount - ns;
    if (rest > 0) {
        const int left = totalStumps - used;
        for (int i = 0; i < rest; ++i) sizes[ns++] = left / rest + (i < left % rest ? 1 : 0);
    }
    int total = 0;
    for (int i = 0; i < stageCount; ++i) total += sizes[i];
    if (total != totalStumps) {
        free(sizes);
        return -1;
    }
    const int64_t npool = vjo_feature_pool(0, WIN, WIN, NULL, 0);
    vjo_feature* pool = (vjo_feature*)malloc(sizeof(vjo_feature) * (size_t)npool);
    vjo_feature_pool(0, WIN, WIN, pool, npool);

    /* calibration windows: face patterns, and texture windows cut at random
     * from two texture scenes (1280x720, 640x360), gated like detection */
    const int nCal = 1000, kNegCal = 8192;
    uint8_t* px = (uint8_t*)malloc((size_t)nCal * WIN * WIN);
    vjo_synth_patches(sm_mix(seed ^ 0xCA11B8A7Eull), nCal, 0, px);
    cal_window* pos = (cal_window*)malloc(sizeof(cal_window) * (size_t)nCal);
    cal_window* neg = (cal_window*)malloc(sizeof(cal_window) * (size_t)kNegCal);
    int npos = 0, nneg = 0;
    for (int i = 0; i < nCal; ++i) {
        cal_ii(px + (size_t)i * WIN * WIN, &pos[npos]);
        if (pos[npos].inv != 0.0f) ++npos;
    }
    {
        const int tw[2] = {1280, 640}, th[2] = {720, 360};
        xo_rng cr = xo_seed(sm_mix(seed ^ 0x7E57u));
        uint8_t win[WIN * WIN];
        for (int t = 0; t < 2; ++t) {
            uint8_t* tex = (uint8_t*)malloc((size_t)tw[t] * th[t]);
            pink(sm_mix(seed + 0x1000u + (uint64_t)t), tw[t], th[t], tex, tw[t]);
            for (int i = 0; i < kNegCal / 2; ++i) {
                const int x0 = xo_range(&cr, 0, tw[t] - WIN);
                const int y0 = xo_range(&cr, 0, th[t] - WIN);
                for (int y = 0; y < WIN; ++y) memcpy(win + y * WIN, tex + (size_t)(y0 + y) * tw[t] + x0, WIN);
                cal_ii(win, &neg[nneg]);
                if (neg[nneg].inv != 0.0f) ++nneg;
            }
            free(tex);
        }
    }

    xo_rng r = xo_seed(sm_mix(seed + 0x5CA5CADEull));
    const int nv = npos + nneg;
    float* vals = (float*)malloc(sizeof(float) * (size_t)(nv > 0 ? nv : 1));
    float* sorted = (float*)malloc(sizeof(float) * (size_t)(nv > 0 ? nv : 1));
    float* negSum = (float*)malloc(sizeof(float) * (size_t)(nneg > 0 ? nneg : 1));
    float* sums = (float*)malloc(sizeof(float) * (size_t)(nneg > 0 ? nneg : 1));
    uint8_t* alive = (uint8_t*)malloc((size_t)(nneg > 0 ? nneg : 1));
    memset(alive, 1, (size_t)(nneg > 0 ? nneg : 1));
    int first = 0;
    for (int si = 0; si < stageCount; ++si) {
        for (int i = 0; i < nneg; ++i) negSum[i] = 0.0f;
        for (int k = 0; k < sizes[si]; ++k) {
            const int fi = (int)(xo_next(&r) % (uint64_t)npool);
            const vjo_feature* f = &pool[fi];
            for (int i = 0; i < npos; ++i) vals[i] = cal_response(f, &pos[i]);
            for (int i = 0; i < nneg; ++i) vals[npos + i] = cal_response(f, &neg[i]);
            memcpy(sorted, vals, sizeof(float) * (size_t)nv);
            qsort(sorted, (size_t)nv, sizeof(float), cmp_float);
            const size_t q = (size_t)xo_range(&r, 300, 700) * (size_t)(nv - 1) / 1000;
            const size_t q1 = q + 1 < (size_t)nv - 1 ? q + 1 : (size_t)nv - 1;
            const float theta = 0.5f * (sorted[q] + sorted[q1]);
            int posRight = 0, negRight = 0;
            for (int i = 0; i < npos; ++i) posRight += vals[i] < theta ? 0 : 1;
            for (int i = 0; i < nneg; ++i) negRight += vals[npos + i] < theta ? 0 : 1;
            const double fp = (double)posRight / (double)npos;
            const double fn = (double)negRight / (double)nneg;
            const double sep = fp - fn;
            const double mag = 0.2 + 4.0 * (sep < 0 ? -sep : sep);
            const float c = (float)(mag < 2.5 ? mag : 2.5);
            const float left = sep >= 0 ? -c : c;
            const float right = sep >= 0 ? c : -c;
            vjo_stump* st = &stumps[first + k];
            const int32_t fbits = fi;
            memcpy(&st->featureBits, &fbits, 4);
            st->theta = theta;
            st->leftVal = left;
            st->rightVal = right;
            for (int i = 0; i < nneg; ++i) negSum[i] += (vals[npos + i] < theta) ? left : right;
        }
        /* the distinct stage sum whose rejection share (sum < threshold) is
         * nearest one half, over the windows alive so far (>= 64) or all */
        int m = 0;
        for (int i = 0; i < nneg; ++i)
            if (alive[i]) sums[m++] = negSum[i];
        if (m < 64) {
            memcpy(sums, negSum, sizeof(float) * (size_t)nneg);
            m = nneg;
        }
        qsort(sums, (size_t)m, sizeof(float), cmp_float);
        float thr = 0.0f;
        if (m > 0) {
            const double half = 0.5 * (double)m;
            double bestGap = 1e300;
            for (int i = 0; i < m; ++i) {
                if (i > 0 && sums[i] == sums[i - 1]) continue;
                const double gap = fabs((double)i - half);
                if (gap < bestGap) {
                    bestGap = gap;
                    thr = sums[i];
                }
            }
        }
        for (int i = 0; i < nneg; ++i)
            if (negSum[i] < thr) alive[i] = 0;
        stages[si].first = first;
        stages[si].ntrees = sizes[si];
        stages[si].threshold = thr;
        first += sizes[si];
    }
    free(sizes);
    free(pool);
    free(px);
    free(pos);
    free(neg);
    free(vals);
    free(sorted);
    free(negSum);
    free(sums);
    free(alive);
    return 0;
}
