/*
 * vj_oracle.c - CPU oracle (test infrastructure; see vj_oracle.h).
 *
 * Plain C restatement of the reference's CPU algorithms for the Viola-Jones
 * data-parallel path.  Compile with -ffp-contract=off.  Citations are to
 * hengyizhu/CS677s26 source files.
 */
#include "vj_oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------ */
/* Haar pool: face_vision_engine.cu:882-1020 (rects from makeFastRect,       */
/* face_vision_engine.cu:618-635).                                           */
/* ------------------------------------------------------------------------ */

static vjo_rect mk_rect(int x, int y, int w, int h, int iiW, float wt, int tilted) {
    vjo_rect r;
    if (!tilted) {
        r.p0 = x + iiW * y;
        r.p1 = (x + w) + iiW * y;
        r.p2 = x + iiW * (y + h);
        r.p3 = (x + w) + iiW * (y + h);
    } else {
        r.p0 = x + iiW * y;
        r.p1 = (x - h) + iiW * (y + h);
        r.p2 = (x + w) + iiW * (y + w);
        r.p3 = (x + w - h) + iiW * (y + w + h);
    }
    r.w = wt;
    return r;
}

typedef struct {
    vjo_feature* out;
    int64_t cap;
    int64_t n;
    int iiW;
} pool_ctx;

static void put(pool_ctx* c, int tilted, int nr, const int* g /* nr x 4 */, const float* wt) {
    if (c->out && c->n < c->cap) {
        vjo_feature f;
        memset(&f, 0, sizeof(f));
        f.r0 = mk_rect(g[0], g[1], g[2], g[3], c->iiW, wt[0], tilted);
        f.r1 = mk_rect(g[4], g[5], g[6], g[7], c->iiW, wt[1], tilted);
        if (nr == 3) f.r2 = mk_rect(g[8], g[9], g[10], g[11], c->iiW, wt[2], tilted);
        f.rectCount = (uint8_t)nr;
        f.tilted = (uint8_t)tilted;
        c->out[c->n] = f;
    }
    c->n++;
}

int64_t vjo_feature_pool(int mode, int W, int H, vjo_feature* out, int64_t cap) {
    pool_ctx c = {out, cap, 0, W + 1};
    const float w2[2] = {-1.0f, 2.0f}, w3[3] = {-1.0f, 2.0f, 2.0f}, w9[2] = {-1.0f, 9.0f};
    const float wt3[2] = {-1.0f, 3.0f};
    for (int x = 0; x < W; ++x)
        for (int y = 0; y < H; ++y)
            for (int dx = 1; dx <= W; ++dx)
                for (int dy = 1; dy <= H; ++dy) {
                    if (x + 2 * dx <= W && y + dy <= H) {
                        int g[8] = {x, y, 2 * dx, dy, x + dx, y, dx, dy};
                        put(&c, 0, 2, g, w2);
                    }
                    if (x + dx <= W && y + 2 * dy <= H) {
                        int g[8] = {x, y, dx, 2 * dy, x, y + dy, dx, dy};
                        put(&c, 0, 2, g, w2);
                    }
                    if (x + 3 * dx <= W && y + dy <= H) {
                        int g[8] = {x, y, 3 * dx, dy, x + dx, y, dx, dy};
                        put(&c, 0, 2, g, w2);
                    }
                    if (x + dx <= W && y + 3 * dy <= H) {
                        int g[8] = {x, y, dx, 3 * dy, x, y + dy, dx, dy};
                        put(&c, 0, 2, g, w2);
                    }
                    if (x + 2 * dx <= W && y + 2 * dy <= H) {
                        int g[12] = {x, y, 2 * dx, 2 * dy, x, y, dx, dy, x + dx, y + dy, dx, dy};
                        put(&c, 0, 3, g, w3);
                    }
                    if (mode >= 1) {
                        if (x + 4 * dx <= W && y + dy <= H) {
                            int g[8] = {x, y, 4 * dx, dy, x + dx, y, 2 * dx, dy};
                            put(&c, 0, 2, g, w2);
                        }
                        if (x + dx <= W && y + 4 * dy <= H) {
                            int g[8] = {x, y, dx, 4 * dy, x, y + dy, dx, 2 * dy};
                            put(&c, 0, 2, g, w2);
                        }
                        if (x + 3 * dx <= W && y + 3 * dy <= H) {
                            int g[8] = {x, y, 3 * dx, 3 * dy, x + dx, y + dy, dx, dy};
                            put(&c, 0, 2, g, w9);
                        }
                    }
                    if (mode >= 2) {
                        if (x + 2 * dx <= W && y + 2 * dx + dy <= H && x - dy >= 0) {
                            int g[8] = {x, y, 2 * dx, dy, x, y, dx, dy};
                            put(&c, 1, 2, g, w2);
                        }
                        if (x + dx <= W && y + dx + 2 * dy <= H && x - 2 * dy >= 0) {
                            int g[8] = {x, y, dx, 2 * dy, x, y, dx, dy};
                            put(&c, 1, 2, g, w2);
                        }
                        if (x + 3 * dx <= W && y + 3 * dx + dy <= H && x - dy >= 0) {
                            int g[8] = {x, y, 3 * dx, dy, x + dx, y + dx, dx, dy};
                            put(&c, 1, 2, g, wt3);
                        }
                        if (x + dx <= W && y + dx + 3 * dy <= H && x - 3 * dy >= 0) {
                            int g[8] = {x, y, dx, 3 * dy, x - dy, y + dy, dx, dy};
                            put(&c, 1, 2, g, wt3);
                        }
                        if (x + 4 * dx <= W && y + 4 * dx + dy <= H && x - dy >= 0) {
                            int g[8] = {x, y, 4 * dx, dy, x + dx, y + dx, 2 * dx, dy};
                            put(&c, 1, 2, g, w2);
                        }
                        if (x + dx <= W && y + dx + 4 * dy <= H && x - 4 * dy >= 0) {
                            int g[8] = {x, y, dx, 4 * dy, x - dy, y + dy, dx, 2 * dy};
                            put(&c, 1, 2, g, w2);
                        }
                    }
                }
    return c.n;
}

/* ------------------------------------------------------------------------ */
/* Integral images: buildHostIntegralImage, main.cu:428-474                  */
/* ------------------------------------------------------------------------ */

void vjo_integral(const uint8_t* gray, int w, int h, int stride, uint32_t* sum, uint64_t* sq) {
    const int iiW = w + 1;
    for (int x = 0; x <= w; ++x) {
        sum[x] = 0;
        sq[x] = 0;
    }
    for (int y = 1; y <= h; ++y) {
        uint32_t rs = 0;
        uint64_t rq = 0;
        sum[(size_t)y * iiW] = 0;
        sq[(size_t)y * iiW] = 0;
        for (int x = 1; x <= w; ++x) {
            const uint32_t p = gray[(size_t)(y - 1) * stride + (x - 1)];
            rs += p;
            rq += (uint64_t)(p * p);
            const size_t i = (size_t)y * iiW + x;
            sum[i] = sum[i - iiW] + rs; /* int32 wrap semantics as uint32 */
            sq[i] = sq[i - iiW] + rq;
        }
    }
}

/* invNorm over the 22x22 interior, main.cu:457-472 / face_vision_engine.cu:216-259:
 * nf2 = area*sq - s^2 in double, invNorm = (float)(1/sqrt(nf2)) or 0. */
static float train_invnorm(const uint32_t* s, const uint64_t* q, int iiW, int iiH) {
    if (iiW < 3 || iiH < 3) return 1.0f;
    const int ww = iiW - 3, hh = iiH - 3, area = ww * hh;
    const int p0 = 1 + iiW, p1 = (1 + ww) + iiW, p2 = 1 + iiW * (1 + hh), p3 = (1 + ww) + iiW * (1 + hh);
    const int32_t si = (int32_t)(s[p0] - s[p1] - s[p2] + s[p3]);
    const int32_t qi = (int32_t)((uint32_t)q[p0] - (uint32_t)q[p1] - (uint32_t)q[p2] + (uint32_t)q[p3]);
    const double sd = (double)si, qd = (double)qi;
    const double nf2 = (double)area * qd - sd * sd;
    return (nf2 > 1e-12) ? (float)(1.0 / sqrt(nf2)) : 0.0f;
}

void vjo_train_integrals(const uint8_t* patches, int n, uint32_t* sums, float* invNorm) {
    uint64_t sq[625];
    for (int i = 0; i < n; ++i) {
        uint32_t* s = sums + (size_t)i * 625;
        vjo_integral(patches + (size_t)i * 576, 24, 24, 24, s, sq);
        invNorm[i] = train_invnorm(s, sq, 25, 25);
    }
}

/* evalTrainingFeatureHost, main.cu:476-496 */
float vjo_train_response(const vjo_feature* f, const uint32_t* s, float invNorm) {
#define RS(r) ((float)(int32_t)s[(r).p0] - (float)(int32_t)s[(r).p1] - (float)(int32_t)s[(r).p2] + \
               (float)(int32_t)s[(r).p3])
    const float s0 = RS(f->r0);
    const float s1 = RS(f->r1);
    float resp = f->r0.w * s0 + f->r1.w * s1;
    if (f->rectCount == 3) {
        const float s2 = RS(f->r2);
        resp += f->r2.w * s2;
    }
#undef RS
    return resp * invNorm;
}

/* ------------------------------------------------------------------------ */
/* Best-weak search: runCpuWeakSearch, main.cu:587-682                       */
/* ------------------------------------------------------------------------ */

typedef struct {
    float v;
    uint16_t i;
} kv;

/* Order of std::stable_sort with the comparator of main.cu:618-624: by value,
 * then by sample index.  -0.0f and +0.0f compare equal. */
static int kv_less(const kv* a, const kv* b) {
    if (a->v < b->v) return 1;
    if (a->v > b->v) return 0;
    return a->i < b->i;
}

static void kv_sort(kv* a, kv* tmp, int n) {
    for (int width = 1; width < n; width *= 2) {
        for (int lo = 0; lo < n; lo += 2 * width) {
            int mid = lo + width < n ? lo + width : n;
            int hi = lo + 2 * width < n ? lo + 2 * width : n;
            int i = lo, j = mid, k = lo;
            while (i < mid && j < hi) tmp[k++] = kv_less(&a[j], &a[i]) ? a[j++] : a[i++];
            while (i < mid) tmp[k++] = a[i++];
            while (j < hi) tmp[k++] = a[j++];
        }
        memcpy(a, tmp, sizeof(kv) * (size_t)n);
    }
}

/* The CPU search's update rule (main.cu:660-677) for candidates of one
 * feature: lower err wins; at equal err parity +1 replaces parity -1. */
static void consider(vjo_best* b, float err, int parity, int k, float theta) {
    if (err < b->err || (err == b->err && parity > b->parity)) {
        b->err = err;
        b->parity = parity;
        b->split = k;
        b->theta = theta;
    }
}

/* Sorted responses of one feature: v[k] and the sample ix[k] at sorted
 * position k (the stable_sort of main.cu:612-624). */
static void sort_feature(const vjo_feature* f, const uint32_t* sums, const float* invNorm, int n, kv* a, kv* t,
                         float* v, uint16_t* ix) {
    for (int i = 0; i < n; ++i) {
        a[i].v = vjo_train_response(f, sums + (size_t)i * 625, invNorm[i]);
        a[i].i = (uint16_t)i;
    }
    kv_sort(a, t, n);
    for (int k = 0; k < n; ++k) {
        v[k] = a[k].v;
        ix[k] = a[k].i;
    }
}

/* Threshold sweep of one feature over its sorted samples, main.cu:626-678:
 * sequential FP32 totals over the sorted order (inactive samples skipped),
 * then the sequential left sums and, at every valid split
 * (v[k] + 1e-7f < v[k+1]), both parities' errors.  b arrives with
 * featureIdx set and err = +inf; *best64 receives the feature's smallest FP64
 * error over its valid splits and b->err64 the FP64 error of the chosen one. */
static void sweep_feature(const float* v, const uint16_t* ix, int n, const int8_t* labels, const uint8_t* active,
                          const float* weights, vjo_best* b, double* best64) {
    float tp = 0.0f, tn = 0.0f;
    double tp64 = 0.0, tn64 = 0.0;
    for (int k = 0; k < n; ++k) {
        const int s = ix[k];
        if (active && active[s] == 0) continue;
        if (labels[s] > 0) {
            tp += weights[s];
            tp64 += (double)weights[s];
        } else {
            tn += weights[s];
            tn64 += (double)weights[s];
        }
    }
    float lp = 0.0f, ln = 0.0f;
    double lp64 = 0.0, ln64 = 0.0, m64 = INFINITY;
    for (int k = 0; k + 1 < n; ++k) {
        const int s = ix[k];
        if (!active || active[s] != 0) {
            if (labels[s] > 0) {
                lp += weights[s];
                lp64 += (double)weights[s];
            } else {
                ln += weights[s];
                ln64 += (double)weights[s];
            }
        }
        const float v0 = v[k], v1 = v[k + 1];
        if (!(v0 + 1e-7f < v1)) continue;
        const float rp = tp - lp, rn = tn - ln;
        const float theta = 0.5f * (v0 + v1);
        const float eL = ln + rp; /* left predicts +1: parity -1 */
        consider(b, eL, -1, k, theta);
        const float eR = lp + rn; /* left predicts -1: parity +1 */
        consider(b, eR, +1, k, theta);
        const double e1 = ln64 + (tp64 - lp64), e2 = lp64 + (tn64 - ln64);
        if (e1 < m64) m64 = e1;
        if (e2 < m64) m64 = e2;
        if (k == b->split) b->err64 = (b->parity < 0) ? e1 : e2;
    }
    *best64 = m64;
}

static vjo_best no_split(int f) {
    vjo_best b;
    b.featureIdx = f;
    b.err = INFINITY;
    b.theta = 0.0f;
    b.parity = 1;
    b.split = -1;
    b.err64 = INFINITY;
    return b;
}

/* A pool's per-feature sorted responses, kept for a stage (see
 * vjo_sorted_build): row f holds v[f][k] and ix[f][k]. */
struct vjo_sorted {
    int nFeat, n;
    float* v;
    uint16_t* ix;
};

typedef struct {
    const vjo_feature* feats;
    const uint8_t* usedMask;
    const uint32_t* sums;
    const float* invNorm;
    const int8_t* labels;
    const uint8_t* active;
    const float* weights;
    int n;
    int f0, f1;
    vjo_best* per;           /* per-feature best, CPU semantics */
    double* err64;           /* per-feature FP64 best (may be NULL) */
    const vjo_sorted* sorted; /* sweep stored orders instead of sorting */
    vjo_sorted* build;       /* fill these rows instead of sweeping */
} search_job;

static void* search_worker(void* arg) {
    search_job* J = (search_job*)arg;
    const int n = J->n;
    kv* a = (kv*)malloc(sizeof(kv) * (size_t)n);
    kv* t = (kv*)malloc(sizeof(kv) * (size_t)n);
    float* v = (float*)malloc(sizeof(float) * (size_t)n);
    uint16_t* ix = (uint16_t*)malloc(sizeof(uint16_t) * (size_t)n);
    for (int f = J->f0; f < J->f1; ++f) {
        if (J->build) {
            sort_feature(&J->feats[f], J->sums, J->invNorm, n, a, t, J->build->v + (size_t)f * n,
                         J->build->ix + (size_t)f * n);
            continue;
        }
        vjo_best b = no_split(f);
        if (J->usedMask && J->usedMask[f]) {
            J->per[f] = b;
            if (J->err64) J->err64[f] = INFINITY;
            continue;
        }
        const float* fv = v;
        const uint16_t* fix = ix;
        if (J->sorted) {
            fv = J->sorted->v + (size_t)f * n;
            fix = J->sorted->ix + (size_t)f * n;
        } else {
            sort_feature(&J->feats[f], J->sums, J->invNorm, n, a, t, v, ix);
        }
        double m64;
        sweep_feature(fv, fix, n, J->labels, J->active, J->weights, &b, &m64);
        J->per[f] = b;
        if (J->err64) J->err64[f] = m64;
    }
    free(a);
    free(t);
    free(v);
    free(ix);
    return NULL;
}

static void run_search(search_job* base, int nFeat, int threads) {
    if (threads < 1) threads = 1;
    if (threads > 256) threads = 256;
    pthread_t tid[256];
    search_job jobs[256];
    const int chunk = (nFeat + threads - 1) / threads;
    int started = 0;
    for (int t = 0; t < threads; ++t) {
        jobs[t] = *base;
        jobs[t].f0 = t * chunk < nFeat ? t * chunk : nFeat;
        jobs[t].f1 = (t + 1) * chunk < nFeat ? (t + 1) * chunk : nFeat;
        if (threads == 1) {
            search_worker(&jobs[t]);
        } else if (pthread_create(&tid[t], NULL, search_worker, &jobs[t]) == 0) {
            started = t + 1;
        } else {
            search_worker(&jobs[t]);
            started = t + 1;
            tid[t] = 0;
        }
    }
    for (int t = 0; t < started; ++t)
        if (threads > 1 && tid[t]) pthread_join(tid[t], NULL);
}

/* Across features, in increasing featureIdx, only a strictly lower err
 * replaces the current best (main.cu:660-662: featureIdx < best.featureIdx
 * never holds for a later feature). */
static vjo_best pick_across(const vjo_best* per, int nFeat) {
    vjo_best g = no_split(-1);
    for (int f = 0; f < nFeat; ++f)
        if (per[f].split >= 0 && per[f].err < g.err) g = per[f];
    return g;
}

void vjo_weak_search(const vjo_feature* feats, int nFeat, const uint8_t* usedMask,
                     const uint32_t* sums, const float* invNorm, const int8_t* labels,
                     const uint8_t* active, const float* weights, int n, int threads,
                     vjo_best* out, vjo_best* perFeature) {
    vjo_best* per = perFeature ? perFeature : (vjo_best*)malloc(sizeof(vjo_best) * (size_t)(nFeat > 0 ? nFeat : 1));
    search_job J = {feats, usedMask, sums, invNorm, labels, active, weights, n, 0, 0, per, NULL, NULL, NULL};
    run_search(&J, nFeat, threads);
    *out = pick_across(per, nFeat);
    if (!perFeature) free(per);
}

void vjo_feature_err64(const vjo_feature* feats, int nFeat, const uint8_t* usedMask,
                       const uint32_t* sums, const float* invNorm, const int8_t* labels,
                       const uint8_t* active, const float* weights, int n, int threads,
                       double* err64) {
    vjo_best* per = (vjo_best*)malloc(sizeof(vjo_best) * (size_t)(nFeat > 0 ? nFeat : 1));
    search_job J = {feats, usedMask, sums, invNorm, labels, active, weights, n, 0, 0, per, err64, NULL, NULL};
    run_search(&J, nFeat, threads);
    free(per);
}

vjo_sorted* vjo_sorted_build(const vjo_feature* feats, int nFeat, const uint32_t* sums, const float* invNorm,
                             int n, int threads) {
    vjo_sorted* s = (vjo_sorted*)calloc(1, sizeof(vjo_sorted));
    if (!s) return NULL;
    s->nFeat = nFeat;
    s->n = n;
    s->v = (float*)malloc(sizeof(float) * (size_t)nFeat * (size_t)n);
    s->ix = (uint16_t*)malloc(sizeof(uint16_t) * (size_t)nFeat * (size_t)n);
    if (!s->v || !s->ix) {
        vjo_sorted_free(s);
        return NULL;
    }
    search_job J = {feats, NULL, sums, invNorm, NULL, NULL, NULL, n, 0, 0, NULL, NULL, NULL, s};
    run_search(&J, nFeat, threads);
    return s;
}

void vjo_sorted_search(const vjo_sorted* s, const uint8_t* usedMask, const int8_t* labels, const uint8_t* active,
                       const float* weights, int threads, vjo_best* out, vjo_best* perFeature) {
    const int nFeat = s->nFeat;
    vjo_best* per = perFeature ? perFeature : (vjo_best*)malloc(sizeof(vjo_best) * (size_t)(nFeat > 0 ? nFeat : 1));
    search_job J = {NULL, usedMask, NULL, NULL, labels, active, weights, s->n, 0, 0, per, NULL, s, NULL};
    run_search(&J, nFeat, threads);
    *out = pick_across(per, nFeat);
    if (!perFeature) free(per);
}

void vjo_sorted_free(vjo_sorted* s) {
    if (!s) return;
    free(s->v);
    free(s->ix);
    free(s);
}

/* ------------------------------------------------------------------------ */
/* Round update (main.cu:2082-2102, 829-906) with FP64 alpha/log and         */
/* renormalisation.                                                          */
/* ------------------------------------------------------------------------ */

void vjo_round_update(const vjo_feature* feats, const vjo_best* best, const uint32_t* sums,
                      const float* invNorm, const int8_t* labels, const uint8_t* active,
                      float* weights, float* strong, int n, float* weakOut) {
    const float eps = 1e-6f;
    float e = best->err;
    if (e < eps) e = eps;
    if (e > 1.0f - eps) e = 1.0f - eps;
    const double ed = (double)e;
    const float C = (float)log((1.0 - ed) / ed);
    const double F = exp((double)C);
    const float left = best->parity > 0 ? -C : C;
    const float right = best->parity > 0 ? C : -C;
    const vjo_feature* f = &feats[best->featureIdx];
    double* x = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    for (int i = 0; i < n; ++i) {
        const float r = vjo_train_response(f, sums + (size_t)i * 625, invNorm[i]);
        const int lt = r < best->theta;
        strong[i] += lt ? left : right;
        if (active && active[i] == 0) {
            x[i] = 0.0;
            continue;
        }
        const int pred = best->parity > 0 ? (lt ? -1 : 1) : (lt ? 1 : -1);
        x[i] = (double)weights[i];
        if (pred != (int)labels[i]) x[i] = x[i] * F;
    }
    double part[1024];
    for (int t = 0; t < 1024; ++t) {
        double s = 0.0;
        for (int i = t; i < n; i += 1024) s += x[i];
        part[t] = s;
    }
    for (int s = 512; s >= 1; s >>= 1)
        for (int t = 0; t < s; ++t) part[t] = part[t] + part[t + s];
    const double Z = part[0];
    for (int i = 0; i < n; ++i) weights[i] = (Z > 1e-30) ? (float)(x[i] / Z) : (float)x[i];
    free(x);
    weakOut[0] = best->theta;
    weakOut[1] = e;
    weakOut[2] = C;
    weakOut[3] = left;
    weakOut[4] = right;
    weakOut[5] = (float)best->parity;
    weakOut[6] = (float)best->featureIdx;
}

/* ------------------------------------------------------------------------ */
/* Stage calibration, main.cu:2168-2300                                      */
/* ------------------------------------------------------------------------ */

static uint32_t radix_key(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

static int cmp_radix(const void* a, const void* b) {
    const uint32_t x = radix_key(*(const float*)a), y = radix_key(*(const float*)b);
    return x < y ? -1 : (x > y ? 1 : 0);
}

void vjo_stage_calibrate(const float* strong, const uint8_t* active, int n, int numPos,
                         float minHitRate, float maxFalseAlarm, int stageNegBase, float* outF,
                         int32_t* outI) {
    const int need = (int)ceilf(minHitRate * (float)numPos);
    const int minPass = need > 1 ? need : 1;
    const int cutIdx = numPos - minPass;
    float* ps = (float*)malloc(sizeof(float) * (size_t)(numPos > 0 ? numPos : 1));
    memcpy(ps, strong, sizeof(float) * (size_t)numPos);
    qsort(ps, (size_t)numPos, sizeof(float), cmp_radix); /* DeviceRadixSort order */
    const float cut = ps[cutIdx];
    free(ps);
    int posGe = 0, posGt = 0, negGe = 0, negGt = 0;
    for (int i = 0; i < n; ++i) {
        const float s = strong[i];
        if (i < numPos) {
            posGe += s >= cut;
            posGt += s > cut;
        } else if (!active || active[i] != 0) {
            negGe += s >= cut;
            negGt += s > cut;
        }
    }
    const int strictGt = posGt >= minPass;
    const float thr = strictGt ? nextafterf(cut, INFINITY) : cut;
    const int posPass = strictGt ? posGt : posGe;
    const int negSurvive = strictGt ? negGt : negGe;
    const float hit = (float)posPass / (float)numPos;
    const float fa = (float)negSurvive / (float)stageNegBase;
    outF[0] = cut;
    outF[1] = thr;
    outF[2] = hit;
    outF[3] = fa;
    outI[0] = strictGt;
    outI[1] = posPass;
    outI[2] = negSurvive;
    outI[3] = (hit >= minHitRate && fa <= maxFalseAlarm) || negSurvive == 0;
}

/* ------------------------------------------------------------------------ */
/* Pyramid resize: resizeGrayBilinearHost, main.cu:545-585                   */
/* ------------------------------------------------------------------------ */

void vjo_resize(const uint8_t* src, int sw, int sh, int ss, uint8_t* dst, int dw, int dh) {
    const float scaleX = (float)sw / (float)dw;
    const float scaleY = (float)sh / (float)dh;
    for (int y = 0; y < dh; ++y) {
        for (int x = 0; x < dw; ++x) {
            const float fx = ((float)x + 0.5f) * scaleX - 0.5f;
            const float fy = ((float)y + 0.5f) * scaleY - 0.5f;
            int sx0 = (int)floorf(fx), sy0 = (int)floorf(fy);
            if (sx0 > sw - 1) sx0 = sw - 1;
            if (sx0 < 0) sx0 = 0;
            if (sy0 > sh - 1) sy0 = sh - 1;
            if (sy0 < 0) sy0 = 0;
            const int sx1 = sx0 + 1 < sw - 1 ? sx0 + 1 : sw - 1;
            const int sy1 = sy0 + 1 < sh - 1 ? sy0 + 1 : sh - 1;
            const float ax = fx - (float)sx0, ay = fy - (float)sy0;
            const float p00 = (float)src[(size_t)sy0 * ss + sx0], p01 = (float)src[(size_t)sy0 * ss + sx1];
            const float p10 = (float)src[(size_t)sy1 * ss + sx0], p11 = (float)src[(size_t)sy1 * ss + sx1];
            const float top = p00 + (p01 - p00) * ax;
            const float bot = p10 + (p11 - p10) * ax;
            const float val = top + (bot - top) * ay;
            int v = (int)(val + 0.5f);
            if (v < 0) v = 0;
            if (v > 255) v = 255;
            dst[(size_t)y * dw + x] = (uint8_t)v;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Multiscale detection: detectMultiScaleCpu, main.cu:684-827                */
/* ------------------------------------------------------------------------ */

typedef struct {
    int dx[3][4], dy[3][4];
    float w[3];
    int nr;
} dec_feature;

typedef struct {
    const dec_feature* dec;
    const vjo_stump* stumps;
    const vjo_stage* stages;
    int nStages;
    const uint32_t* sum;
    const uint64_t* sq;
    int iiW;
    int winW, winH, workW, workH, step;
    int normMode;
    float scale;
    int scaleIdx;
    int y0, y1; /* rows [y0, y1) of window origins, multiples of step */
    vjo_det* out;
    int cap, count;
} det_job;

static inline float corner(const uint32_t* s, int p) { return (float)(int32_t)s[p]; }

static void* detect_rows(void* arg) {
    det_job* J = (det_job*)arg;
    const int iiW = J->iiW;
    const int nw = J->winW - 2, nh = J->winH - 2, narea = nw * nh;
    const int np0 = 1 + iiW, np1 = (1 + nw) + iiW, np2 = 1 + iiW * (1 + nh), np3 = (1 + nw) + iiW * (1 + nh);
    J->count = 0;
    for (int y = J->y0; y < J->y1; y += J->step) {
        for (int x = 0; x < J->workW; x += J->step) {
            const int b = y * iiW + x;
            double normSum;
            if (J->normMode == 0) {
                normSum = (double)(corner(J->sum, b + np0) - corner(J->sum, b + np1) -
                                   corner(J->sum, b + np2) + corner(J->sum, b + np3));
            } else {
                normSum = (double)(int32_t)(J->sum[b + np0] - J->sum[b + np1] - J->sum[b + np2] +
                                            J->sum[b + np3]);
            }
            const uint32_t nq = (uint32_t)J->sq[b + np0] - (uint32_t)J->sq[b + np1] -
                                (uint32_t)J->sq[b + np2] + (uint32_t)J->sq[b + np3];
            const double nf2 = (double)narea * (double)nq - normSum * normSum;
            if (!(nf2 > 0.0)) continue;
            const float inv = (float)(1.0 / sqrt(nf2));
            if (!((double)narea * (double)inv < 1e-1)) continue;
            int pass = 1;
            float last = 0.0f;
            for (int si = 0; si < J->nStages; ++si) {
                const vjo_stage st = J->stages[si];
                float stageSum = 0.0f;
                for (int k = 0; k < st.ntrees; ++k) {
                    const vjo_stump sp = J->stumps[st.first + k];
                    int32_t fi;
                    memcpy(&fi, &sp.featureBits, 4);
                    const dec_feature* d = &J->dec[fi];
                    float raw = 0.0f;
                    for (int r = 0; r < d->nr; ++r) {
                        const float v = (corner(J->sum, b + d->dy[r][0] * iiW + d->dx[r][0]) -
                                         corner(J->sum, b + d->dy[r][1] * iiW + d->dx[r][1]) -
                                         corner(J->sum, b + d->dy[r][2] * iiW + d->dx[r][2]) +
                                         corner(J->sum, b + d->dy[r][3] * iiW + d->dx[r][3])) * d->w[r];
                        raw = (r == 0) ? v : raw + v;
                    }
                    const float resp = raw * inv;
                    stageSum += (resp < sp.theta) ? sp.leftVal : sp.rightVal;
                }
                if (stageSum < st.threshold) {
                    pass = 0;
                    break;
                }
                last = stageSum;
            }
            if (pass && J->count < J->cap) {
                vjo_det d;
                d.x = (int)((float)x * J->scale + 0.5f);
                d.y = (int)((float)y * J->scale + 0.5f);
                d.w = (int)((float)J->winW * J->scale + 0.5f);
                d.h = (int)((float)J->winH * J->scale + 0.5f);
                d.scaleIdx = J->scaleIdx;
                d.score = last;
                J->out[J->count++] = d;
            }
        }
    }
    return NULL;
}

int vjo_detect(const vjo_feature* feats, int nFeat, const vjo_stump* stumps, int nStumps,
               const vjo_stage* stages, int nStages, int winW, int winH, const uint8_t* image,
               int w, int h, int stride, float sf, int minObj, int maxDet, int maxScales,
               int normMode, int threads, vjo_det* out, int cap) {
    (void)nStumps;
    const int mW = winW + 1;
    dec_feature* dec = (dec_feature*)calloc((size_t)(nFeat > 0 ? nFeat : 1), sizeof(dec_feature));
    for (int i = 0; i < nFeat; ++i) {
        const vjo_rect* rr[3] = {&feats[i].r0, &feats[i].r1, &feats[i].r2};
        dec[i].nr = feats[i].rectCount == 3 ? 3 : 2;
        for (int r = 0; r < 3; ++r) {
            const int32_t p[4] = {rr[r]->p0, rr[r]->p1, rr[r]->p2, rr[r]->p3};
            for (int c = 0; c < 4; ++c) {
                dec[i].dy[r][c] = p[c] / mW;
                dec[i].dx[r][c] = p[c] - dec[i].dy[r][c] * mW;
            }
            dec[i].w[r] = rr[r]->w;
        }
    }
    if (threads < 1) threads = 1;
    if (threads > 64) threads = 64;
    int total = 0;
    float scale = 1.0f;
    int scaleIdx = 0;
    const uint8_t* prev = image;
    int prevW = w, prevH = h, prevS = stride;
    uint8_t* prevBuf = NULL;
    int done = 0;
    while (!done) {
        if (maxScales > 0 && scaleIdx >= maxScales) break;
        const int sw = (int)roundf((float)w / scale), sh = (int)roundf((float)h / scale);
        const int ow = (int)roundf((float)winW * scale), oh = (int)roundf((float)winH * scale);
        if (sw < winW || sh < winH) break;
        if (ow < minObj || oh < minObj) {
            scale *= sf;
            ++scaleIdx;
            continue;
        }
        const uint8_t* cur;
        int curS;
        uint8_t* buf = NULL;
        if (scaleIdx == 0) {
            cur = image;
            curS = stride;
        } else {
            buf = (uint8_t*)malloc((size_t)sw * sh);
            vjo_resize(prev, prevW, prevH, prevS, buf, sw, sh);
            cur = buf;
            curS = sw;
            free(prevBuf);
            prevBuf = buf;
            prev = buf;
            prevW = sw;
            prevH = sh;
            prevS = sw;
        }
        uint32_t* sum = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(sw + 1) * (sh + 1));
        uint64_t* sq = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)(sw + 1) * (sh + 1));
        vjo_integral(cur, sw, sh, curS, sum, sq);
        const int workW = sw - winW + 1, workH = sh - winH + 1;
        const int step = (scale >= 3.0f) ? 3 : ((scale >= 2.0f) ? 2 : 1);
        const int rows = (workH + step - 1) / step;
        int T = threads < rows ? threads : rows;
        if (T < 1) T = 1;
        det_job jobs[64];
        pthread_t tid[64];
        int ok[64];
        for (int t = 0; t < T; ++t) {
            det_job* J = &jobs[t];
            J->dec = dec;
            J->stumps = stumps;
            J->stages = stages;
            J->nStages = nStages;
            J->sum = sum;
            J->sq = sq;
            J->iiW = sw + 1;
            J->winW = winW;
            J->winH = winH;
            J->workW = workW;
            J->workH = workH;
            J->step = step;
            J->normMode = normMode;
            J->scale = scale;
            J->scaleIdx = scaleIdx;
            J->y0 = (int)((int64_t)rows * t / T) * step;
            J->y1 = (int)((int64_t)rows * (t + 1) / T) * step;
            if (J->y1 > workH) J->y1 = workH;
            J->cap = maxDet - total;
            if (J->cap < 0) J->cap = 0;
            J->out = (vjo_det*)malloc(sizeof(vjo_det) * (size_t)(J->cap > 0 ? J->cap : 1));
            ok[t] = 0;
            if (T > 1 && pthread_create(&tid[t], NULL, detect_rows, J) == 0) ok[t] = 1;
            else detect_rows(J);
        }
        for (int t = 0; t < T; ++t) {
            if (ok[t]) pthread_join(tid[t], NULL);
        }
        for (int t = 0; t < T; ++t) {
            for (int k = 0; k < jobs[t].count && total < maxDet; ++k) {
                if (total < cap) out[total] = jobs[t].out[k];
                ++total;
            }
            free(jobs[t].out);
        }
        free(sum);
        free(sq);
        if (total >= maxDet) done = 1;
        scale *= sf;
        ++scaleIdx;
    }
    free(prevBuf);
    free(dec);
    return total < cap ? total : cap;
}

/* ------------------------------------------------------------------------ */
/* groupRectanglesCpu, face_vision_engine.cu:1401-1539 (union-find with      */
/* path compression and union by rank, face_vision_engine.cu:585-606;        */
/* similarRects :608-616)                                                    */
/* ------------------------------------------------------------------------ */

static int dsu_find(int* p, int x) {
    while (p[x] != x) {
        /* full path compression, as the recursive find does */
        int r = x;
        while (p[r] != r) r = p[r];
        while (p[x] != r) {
            int nx = p[x];
            p[x] = r;
            x = nx;
        }
        return r;
    }
    return x;
}

static void dsu_unite(int* p, int* rk, int a, int b) {
    a = dsu_find(p, a);
    b = dsu_find(p, b);
    if (a == b) return;
    if (rk[a] < rk[b]) {
        int t = a;
        a = b;
        b = t;
    }
    p[b] = a;
    if (rk[a] == rk[b]) ++rk[a];
}

static int similar(const vjo_det* a, const vjo_det* b, float eps) {
    const int mw = a->w < b->w ? a->w : b->w, mh = a->h < b->h ? a->h : b->h;
    const int delta = (int)(eps * (float)(mw + mh) * 0.5f);
    return abs(a->x - b->x) <= delta && abs(a->y - b->y) <= delta &&
           abs((a->x + a->w) - (b->x + b->w)) <= delta && abs((a->y + a->h) - (b->y + b->h)) <= delta;
}

static const vjo_det* g_sort_base;
static int cmp_x_then_index(const void* pa, const void* pb) {
    const int a = *(const int*)pa, b = *(const int*)pb;
    if (g_sort_base[a].x != g_sort_base[b].x) return g_sort_base[a].x < g_sort_base[b].x ? -1 : 1;
    return a < b ? -1 : (a > b ? 1 : 0);
}

/* groupRectanglesCpu; when `first` is given it receives, per output cluster,
 * the smallest input index among the cluster's members. */
static int group_impl(const vjo_det* in, int n, int minNeighbors, float eps, vjo_det* out, int* first) {
    if (n <= 0) return 0;
    int* p = (int*)malloc(sizeof(int) * (size_t)n);
    int* rk = (int*)calloc((size_t)n, sizeof(int));
    int* order = (int*)malloc(sizeof(int) * (size_t)n);
    for (int i = 0; i < n; ++i) {
        p[i] = i;
        order[i] = i;
    }
    g_sort_base = in;
    qsort(order, (size_t)n, sizeof(int), cmp_x_then_index);
    for (int oi = 0; oi < n; ++oi) {
        const int i = order[oi];
        const vjo_det* a = &in[i];
        /* delta computed in float: (int)(eps * float(w + h) * 0.5f) */
        const int maxDx = (int)(eps * (float)(a->w + a->h) * 0.5f);
        for (int oj = oi + 1; oj < n; ++oj) {
            const int j = order[oj];
            if (in[j].x - a->x > maxDx) break;
            if (similar(a, &in[j], eps)) dsu_unite(p, rk, i, j);
        }
    }
    int64_t* sx = (int64_t*)calloc((size_t)n, sizeof(int64_t));
    int64_t* sy = (int64_t*)calloc((size_t)n, sizeof(int64_t));
    int64_t* sw = (int64_t*)calloc((size_t)n, sizeof(int64_t));
    int64_t* sh = (int64_t*)calloc((size_t)n, sizeof(int64_t));
    int* cnt = (int*)calloc((size_t)n, sizeof(int));
    float* bs = (float*)malloc(sizeof(float) * (size_t)n);
    int* bsi = (int*)calloc((size_t)n, sizeof(int));
    int* fst = (int*)malloc(sizeof(int) * (size_t)n);
    for (int i = 0; i < n; ++i) {
        bs[i] = -INFINITY;
        fst[i] = -1;
    }
    for (int i = 0; i < n; ++i) {
        const int r = dsu_find(p, i);
        if (fst[r] < 0) fst[r] = i;
        sx[r] += in[i].x;
        sy[r] += in[i].y;
        sw[r] += in[i].w;
        sh[r] += in[i].h;
        cnt[r] += 1;
        if (in[i].score > bs[r]) {
            bs[r] = in[i].score;
            bsi[r] = in[i].scaleIdx;
        }
    }
    vjo_det* cl = (vjo_det*)malloc(sizeof(vjo_det) * (size_t)n);
    int* cc = (int*)malloc(sizeof(int) * (size_t)n);
    int* cf = (int*)malloc(sizeof(int) * (size_t)n);
    int m = 0;
    const int minN = minNeighbors > 1 ? minNeighbors : 1;
    for (int i = 0; i < n; ++i) {
        if (dsu_find(p, i) != i || cnt[i] <= 0) continue;
        if (cnt[i] <= minN) continue;
        vjo_det d;
        d.x = (int)(sx[i] / cnt[i]);
        d.y = (int)(sy[i] / cnt[i]);
        d.w = (int)(sw[i] / cnt[i]);
        d.h = (int)(sh[i] / cnt[i]);
        d.scaleIdx = bsi[i];
        d.score = bs[i];
        cl[m] = d;
        cc[m] = cnt[i];
        cf[m] = fst[i];
        ++m;
    }
    int maxW = 0;
    for (int i = 0; i < m; ++i)
        if (cl[i].w > maxW) maxW = cl[i].w;
    int* co = (int*)malloc(sizeof(int) * (size_t)(m > 0 ? m : 1));
    for (int i = 0; i < m; ++i) co[i] = i;
    g_sort_base = cl;
    qsort(co, (size_t)m, sizeof(int), cmp_x_then_index);
    int k = 0;
    for (int i = 0; i < m; ++i) {
        const vjo_det* r1 = &cl[i];
        const int n1 = cc[i];
        int discard = 0;
        const float lb = (float)(r1->x + r1->w) - (1.0f + eps) * (float)maxW;
        const float rb = (float)r1->x + eps * (float)maxW;
        for (int q = 0; q < m; ++q) {
            const int o = co[q];
            const vjo_det* r2 = &cl[o];
            if (r2->x < (int)lb) continue;
            if (r2->x > (int)rb) break;
            if (o == i) continue;
            const int n2 = cc[o];
            const int dx = (int)((float)r2->w * eps), dy = (int)((float)r2->h * eps);
            const int big = n1 > 3 ? n1 : 3;
            if (r1->x >= r2->x - dx && r1->y >= r2->y - dy && r1->x + r1->w <= r2->x + r2->w + dx &&
                r1->y + r1->h <= r2->y + r2->h + dy && (n2 > big || n1 < 3)) {
                discard = 1;
                break;
            }
        }
        if (!discard) {
            if (first) first[k] = cf[i];
            out[k++] = *r1;
        }
    }
    free(p);
    free(rk);
    free(order);
    free(sx);
    free(sy);
    free(sw);
    free(sh);
    free(cnt);
    free(bs);
    free(bsi);
    free(fst);
    free(cl);
    free(cc);
    free(cf);
    free(co);
    return k;
}

int vjo_group(const vjo_det* in, int n, int minNeighbors, float eps, vjo_det* out) {
    return group_impl(in, n, minNeighbors, eps, out, NULL);
}

/* The same clusters ordered by their first member's input index (the
 * library's device grouping order when the input is in canonical order). */
int vjo_group_first_order(const vjo_det* in, int n, int minNeighbors, float eps, vjo_det* out) {
    if (n <= 0) return 0;
    vjo_det* tmp = (vjo_det*)malloc(sizeof(vjo_det) * (size_t)n);
    int* first = (int*)malloc(sizeof(int) * (size_t)n);
    const int k = group_impl(in, n, minNeighbors, eps, tmp, first);
    /* insertion by first index: the first indices are distinct */
    int* pos = (int*)malloc(sizeof(int) * (size_t)(k > 0 ? k : 1));
    for (int i = 0; i < k; ++i) pos[i] = i;
    for (int i = 1; i < k; ++i) {
        const int v = pos[i];
        int j = i - 1;
        while (j >= 0 && first[pos[j]] > first[v]) {
            pos[j + 1] = pos[j];
            --j;
        }
        pos[j + 1] = v;
    }
    for (int i = 0; i < k; ++i) out[i] = tmp[pos[i]];
    free(tmp);
    free(first);
    free(pos);
    return k;
}

/* ------------------------------------------------------------------------ */
/* cropResizeTo24: main.cu:245-284.  Every operation is one IEEE single      */
/* rounding in the reference's order (compiled with -ffp-contract=off).      */
/* ------------------------------------------------------------------------ */

void vjo_crop_resize(const uint8_t* img, int w, int h, int stride, int x, int y, int bw, int bh, int out,
                     uint8_t* dst) {
    const float sx = (float)(bw > 1 ? bw : 1);
    const float sy = (float)(bh > 1 ? bh : 1);
    const float stepX = sx / (float)out, stepY = sy / (float)out;
    for (int oy = 0; oy < out; ++oy) {
        for (int ox = 0; ox < out; ++ox) {
            const float fx = (float)x + ((float)ox + 0.5f) * stepX - 0.5f;
            const float fy = (float)y + ((float)oy + 0.5f) * stepY - 0.5f;
            int x0 = (int)floorf(fx), y0 = (int)floorf(fy);
            x0 = x0 < 0 ? 0 : (x0 > w - 1 ? w - 1 : x0);
            y0 = y0 < 0 ? 0 : (y0 > h - 1 ? h - 1 : y0);
            const int x1 = x0 + 1 < w - 1 ? x0 + 1 : w - 1;
            const int y1 = y0 + 1 < h - 1 ? y0 + 1 : h - 1;
            const float ax = fx - (float)x0, ay = fy - (float)y0;
            const float p00 = (float)img[(size_t)y0 * stride + x0], p01 = (float)img[(size_t)y0 * stride + x1];
            const float p10 = (float)img[(size_t)y1 * stride + x0], p11 = (float)img[(size_t)y1 * stride + x1];
            const float top = p00 + (p01 - p00) * ax;
            const float bot = p10 + (p11 - p10) * ax;
            const float val = top + (bot - top) * ay;
            int v = (int)(val + 0.5f);
            v = v < 0 ? 0 : (v > 255 ? 255 : v);
            dst[(size_t)oy * out + ox] = (uint8_t)v;
        }
    }
}
