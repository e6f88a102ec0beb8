// Seeded synthetic inputs: face-like 24x24 patches, 1/f texture patches and
// scenes with pasted face patterns, and a synthetic cascade.  They stand in
// for the Kaggle faces, COCO negatives and demo images that the reference
// trains and detects on (scripts/prepare_data.py, scripts/stage_negatives.py),
// none of which exist offline.
//
// Everything is integer arithmetic or single IEEE operations (+ - * / sqrt,
// compiled without FMA contraction), so the bytes are identical on every
// machine; no libm transcendental function is called.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "common.h"

namespace vjgb {
namespace {

uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// xoshiro256** seeded through splitmix64.
struct Rng {
    uint64_t s[4];
    explicit Rng(uint64_t seed) {
        uint64_t z = seed;
        for (auto& v : s) {
            z += 0x9E3779B97F4A7C15ull;
            v = mix64(z);
        }
    }
    static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    uint64_t next() {
        const uint64_t r = rotl(s[1] * 5, 7) * 9;
        const uint64_t t = s[1] << 17;
        s[2] ^= s[0];
        s[3] ^= s[1];
        s[1] ^= s[2];
        s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return r;
    }
    // Uniform integer in [lo, hi].
    int range(int lo, int hi) {
        const uint64_t span = static_cast<uint64_t>(hi - lo) + 1;
        return lo + static_cast<int>(next() % span);
    }
    // Uniform double in [0, 1) with 53 random bits.
    double unit() { return static_cast<double>(next() >> 11) * (1.0 / 9007199254740992.0); }
    // Approximately Gaussian integer (Irwin-Hall of four 16-bit uniforms)
    // with standard deviation `sigma`.
    int gauss(int sigma) {
        const uint64_t r = next();
        const int64_t s = static_cast<int64_t>(r & 0xFFFF) + static_cast<int64_t>((r >> 16) & 0xFFFF) +
                          static_cast<int64_t>((r >> 32) & 0xFFFF) + static_cast<int64_t>(r >> 48);
        // mean 131070, std 37837.2 -> scale by sigma / 37837.2
        return static_cast<int>(((s * 2 - 262140) * sigma) / 75674);
    }
};

inline int64_t floor_div(int64_t a, int64_t b) {
    int64_t q = a / b;
    if ((a % b != 0) && ((a < 0) != (b < 0))) --q;
    return q;
}

inline uint8_t clamp_u8(int64_t v) { return static_cast<uint8_t>(v < 0 ? 0 : (v > 255 ? 255 : v)); }

// r^t for t = k / 1024, from ten repeated square roots (each correctly
// rounded), so the result is reproducible bit for bit.
double pow_frac1024(double r, int k) {
    double roots[10];
    double v = r;
    for (int j = 0; j < 10; ++j) {
        v = std::sqrt(v);
        roots[j] = v;  // r^(2^-(j+1))
    }
    double out = 1.0;
    for (int j = 0; j < 10; ++j)
        if (k & (512 >> j)) out *= roots[j];
    if (k >= 1024) out *= r;
    return out;
}

// Log-uniform integer in [lo, hi].
int log_uniform(Rng& rng, int lo, int hi) {
    const int k = rng.range(0, 1024);
    const double v = static_cast<double>(lo) * pow_frac1024(static_cast<double>(hi) / lo, k);
    int out = static_cast<int>(std::floor(v + 0.5));
    return std::min(hi, std::max(lo, out));
}

// Value noise summed over octaves of equal amplitude: every octave band then
// carries the same power, which is a 1/f amplitude spectrum (pink noise, scale
// invariant like natural texture).  Scaled to mean 110 and std 45.
void texture(uint64_t seed, int w, int h, uint8_t* out, int stride) {
    const int64_t npx = static_cast<int64_t>(w) * h;
    std::vector<int32_t> acc(static_cast<size_t>(npx), 0);
    const int maxCell = std::min(256, std::max(2, std::max(w, h)));
    Rng orng(seed ^ 0x5eed7e47u);
    std::vector<int32_t> grid;
    for (int cell = 2, oct = 0; cell <= maxCell; cell *= 2, ++oct) {
        const int offx = orng.range(0, cell - 1);
        const int offy = orng.range(0, cell - 1);
        const uint64_t oseed = mix64(seed * 0x100000001B3ull + static_cast<uint64_t>(oct));
        // Lattice values on a (gw x gh) grid covering the image at this octave.
        const int gw = (w - 1 + offx) / cell + 2;
        const int gh = (h - 1 + offy) / cell + 2;
        grid.resize(static_cast<size_t>(gw) * gh);
        for (int gy = 0; gy < gh; ++gy)
            for (int gx = 0; gx < gw; ++gx) {
                const uint64_t hsh = mix64(oseed ^ (static_cast<uint64_t>(gx) * 0xC2B2AE3D27D4EB4Full) ^
                                           (static_cast<uint64_t>(gy) * 0x165667B19E3779F9ull));
                grid[static_cast<size_t>(gy) * gw + gx] = static_cast<int32_t>(hsh & 0xFFFF) - 32768;
            }
        const int64_t c2 = static_cast<int64_t>(cell) * cell;
        for (int y = 0; y < h; ++y) {
            const int iy = (y + offy) / cell;
            const int64_t fy = (y + offy) - static_cast<int64_t>(iy) * cell;
            const int32_t* g0 = grid.data() + static_cast<size_t>(iy) * gw;
            const int32_t* g1 = g0 + gw;
            int32_t* arow = acc.data() + static_cast<size_t>(y) * w;
            for (int x = 0; x < w; ++x) {
                const int ix = (x + offx) / cell;
                const int64_t fx = (x + offx) - static_cast<int64_t>(ix) * cell;
                const int64_t top = static_cast<int64_t>(g0[ix]) * (cell - fx) + static_cast<int64_t>(g0[ix + 1]) * fx;
                const int64_t bot = static_cast<int64_t>(g1[ix]) * (cell - fx) + static_cast<int64_t>(g1[ix + 1]) * fx;
                const int64_t v = floor_div(top * (cell - fy) + bot * fy, c2);
                arow[x] += static_cast<int32_t>(v);
            }
        }
    }
    double sum = 0.0;
    for (int64_t i = 0; i < npx; ++i) sum += static_cast<double>(acc[static_cast<size_t>(i)]);
    const double mean = sum / static_cast<double>(npx);
    double ss = 0.0;
    for (int64_t i = 0; i < npx; ++i) {
        const double d = static_cast<double>(acc[static_cast<size_t>(i)]) - mean;
        ss += d * d;
    }
    double sd = std::sqrt(ss / static_cast<double>(npx));
    if (!(sd > 0.0)) sd = 1.0;
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
            const double d = static_cast<double>(acc[static_cast<size_t>(y) * w + x]) - mean;
            const double v = 110.0 + 45.0 * (d / sd);
            out[static_cast<size_t>(y) * stride + x] = clamp_u8(static_cast<int64_t>(std::floor(v + 0.5)));
        }
}

// One face-like 24x24 pattern: texture background, an ellipse with a vertical
// brightness gradient around mean 140, two darker eye ellipses (-50), a mouth
// band (-35) and Gaussian noise of sigma 12, clipped to 0..255.  Geometry is in
// quarter-pixel units so every test is an integer comparison.
void face(Rng& rng, uint8_t* p) {
    texture(rng.next(), kWin, kWin, p, kWin);
    const int cx = 4 * 12 + rng.range(-4, 4);
    const int cy = 4 * 12 + rng.range(-4, 4);
    const int a = 4 * 9 + rng.range(-3, 3);   // horizontal semi-axis
    const int b = 4 * 11 + rng.range(-3, 3);  // vertical semi-axis
    const int grad = rng.range(-15, 15);
    const int eyeDx = 4 * 4 + rng.range(-2, 2);
    const int eyeDy = 4 * 3 + rng.range(-2, 2);
    const int ea = 10, eb = 6;
    const int64_t a2 = static_cast<int64_t>(a) * a, b2 = static_cast<int64_t>(b) * b;
    for (int y = 0; y < kWin; ++y) {
        for (int x = 0; x < kWin; ++x) {
            const int px = 4 * x + 2, py = 4 * y + 2;
            const int dx = px - cx, dy = py - cy;
            int v = p[y * kWin + x];
            if (static_cast<int64_t>(dx) * dx * b2 + static_cast<int64_t>(dy) * dy * a2 <= a2 * b2) {
                v = 140 + (grad * dy) / b;
                for (int side = -1; side <= 1; side += 2) {
                    const int ex = dx - side * eyeDx, ey = dy + eyeDy;
                    if (ex * ex * eb * eb + ey * ey * ea * ea <= ea * ea * eb * eb) v -= 50;
                }
                if (dx >= -16 && dx <= 16 && dy >= 16 && dy < 24) v -= 35;
            }
            v += rng.gauss(12);
            p[y * kWin + x] = clamp_u8(v);
        }
    }
}

// Bilinear resize of a 24x24 pattern to s x s (pixel-centre geometry, 16.16
// fixed point), written at (x0, y0) of a w-wide scene.
void paste(const uint8_t* src, int s, uint8_t* dst, int stride, int x0, int y0) {
    for (int y = 0; y < s; ++y) {
        const int64_t fy = ((2LL * y + 1) * kWin * 65536) / (2LL * s) - 32768;
        int64_t sy = floor_div(fy, 65536);
        int64_t ay = fy - sy * 65536;
        if (sy < 0) { sy = 0; ay = 0; }
        if (sy >= kWin - 1) { sy = kWin - 1; ay = 0; }
        const int64_t sy1 = std::min<int64_t>(sy + 1, kWin - 1);
        for (int x = 0; x < s; ++x) {
            const int64_t fx = ((2LL * x + 1) * kWin * 65536) / (2LL * s) - 32768;
            int64_t sx = floor_div(fx, 65536);
            int64_t ax = fx - sx * 65536;
            if (sx < 0) { sx = 0; ax = 0; }
            if (sx >= kWin - 1) { sx = kWin - 1; ax = 0; }
            const int64_t sx1 = std::min<int64_t>(sx + 1, kWin - 1);
            const int64_t p00 = src[sy * kWin + sx], p01 = src[sy * kWin + sx1];
            const int64_t p10 = src[sy1 * kWin + sx], p11 = src[sy1 * kWin + sx1];
            const int64_t top = p00 * (65536 - ax) + p01 * ax;
            const int64_t bot = p10 * (65536 - ax) + p11 * ax;
            const int64_t v = (top * (65536 - ay) + bot * ay + (1LL << 31)) >> 32;
            dst[static_cast<size_t>(y0 + y) * stride + (x0 + x)] = clamp_u8(v);
        }
    }
}

// ---- host feature arithmetic used only to calibrate the synthetic cascade ----
struct PatchII {
    int32_t sum[kIIArea];
    float invNorm;  // detection-style window normalisation; 0 = window gated out
};

void patch_ii(const uint8_t* p, PatchII* out) {
    int64_t sq[kIIArea];
    for (int i = 0; i < kIIArea; ++i) { out->sum[i] = 0; sq[i] = 0; }
    for (int y = 1; y <= kWin; ++y) {
        int32_t rs = 0;
        int64_t rq = 0;
        for (int x = 1; x <= kWin; ++x) {
            const int v = p[(y - 1) * kWin + (x - 1)];
            rs += v;
            rq += v * v;
            out->sum[y * kIIW + x] = out->sum[(y - 1) * kIIW + x] + rs;
            sq[y * kIIW + x] = sq[(y - 1) * kIIW + x] + rq;
        }
    }
    const int q0 = 1 * kIIW + 1, q1 = 1 * kIIW + 23, q2 = 23 * kIIW + 1, q3 = 23 * kIIW + 23;
    const double s = static_cast<double>(out->sum[q0] - out->sum[q1] - out->sum[q2] + out->sum[q3]);
    const double ss = static_cast<double>(sq[q0] - sq[q1] - sq[q2] + sq[q3]);
    const double nf2 = 484.0 * ss - s * s;
    out->invNorm = 0.0f;
    if (nf2 > 0.0) {
        const float inv = static_cast<float>(1.0 / std::sqrt(nf2));
        if (484.0 * static_cast<double>(inv) < 0.1) out->invNorm = inv;
    }
}

float patch_response(const vj_haar_feature& f, const PatchII& ii) {
    auto rect = [&](const vj_fast_rect& r) {
        return (static_cast<float>(ii.sum[r.p0]) - static_cast<float>(ii.sum[r.p1]) -
                static_cast<float>(ii.sum[r.p2]) + static_cast<float>(ii.sum[r.p3])) * r.w;
    };
    float raw = rect(f.r0) + rect(f.r1);
    if (f.rectCount == 3) raw += rect(f.r2);
    return raw * ii.invNorm;
}

}  // namespace
}  // namespace vjgb

using namespace vjgb;

extern "C" {

int vj_synth_patches(uint64_t seed, int nPos, int nNeg, uint8_t* out) {
    if (!out || nPos < 0 || nNeg < 0) return set_error(VJ_INVALID_ARG, "vj_synth_patches: bad arguments");
    const size_t px = static_cast<size_t>(kWin) * kWin;
    for (int i = 0; i < nPos; ++i) {
        Rng rng(mix64(seed * 0x9E3779B97F4A7C15ull + 0x1000000ull + static_cast<uint64_t>(i)));
        face(rng, out + static_cast<size_t>(i) * px);
    }
    for (int i = 0; i < nNeg; ++i) {
        const uint64_t s = mix64(seed * 0x9E3779B97F4A7C15ull + 0x2000000000ull + static_cast<uint64_t>(i));
        texture(s, kWin, kWin, out + static_cast<size_t>(nPos + i) * px, kWin);
    }
    return ok();
}

int vj_synth_scene(uint64_t seed, int w, int h, int nPaste, int minSize, int maxSize, uint8_t* out) {
    if (!out || w < kWin || h < kWin || nPaste < 0 || minSize < 1 || maxSize < minSize)
        return set_error(VJ_INVALID_ARG, "vj_synth_scene: bad arguments");
    texture(mix64(seed ^ 0xA5A5A5A5ull), w, h, out, w);
    Rng rng(mix64(seed + 0x3C3C3C3Cull));
    uint8_t pat[kWin * kWin];
    const int smax = std::min(maxSize, std::min(w, h));
    const int smin = std::min(minSize, smax);
    for (int k = 0; k < nPaste; ++k) {
        const int s = log_uniform(rng, smin, smax);
        const int x0 = rng.range(0, w - s);
        const int y0 = rng.range(0, h - s);
        Rng frng(rng.next());
        face(frng, pat);
        paste(pat, s, out, w, x0, y0);
    }
    return ok();
}

int vj_synth_cascade(uint64_t seed, int stageCount, int totalStumps, vj_stump4* stumps,
                     vj_cascade_stage* stages) {
    const int head[5] = {1, 10, 25, 25, 50};
    if (!stumps || !stages || stageCount < 1 || totalStumps < stageCount)
        return set_error(VJ_INVALID_ARG, "vj_synth_cascade: bad arguments");
    // Stage sizes: the first five fixed, the remainder spread evenly with the
    // larger shares first (6061 over 38 stages: 1,10,25,25,50, 10x181, 23x180).
    std::vector<int> sizes;
    int used = 0;
    for (int i = 0; i < stageCount && i < 5; ++i) {
        const int take = std::min(head[i], totalStumps - used - (stageCount - i - 1));
        sizes.push_back(std::max(1, take));
        used += sizes.back();
    }
    const int rest = stageCount - static_cast<int>(sizes.size());
    if (rest > 0) {
        const int left = totalStumps - used;
        for (int i = 0; i < rest; ++i) sizes.push_back(left / rest + (i < left % rest ? 1 : 0));
    }
    int total = 0;
    for (int s : sizes) total += s;
    if (total != totalStumps) return set_error(VJ_INVALID_ARG, "vj_synth_cascade: sizes do not add up");

    std::vector<vj_haar_feature> pool(static_cast<size_t>(build_feature_pool(VJ_FEATURES_BASIC, kWin, kWin, nullptr, 0)));
    build_feature_pool(VJ_FEATURES_BASIC, kWin, kWin, pool.data(), static_cast<int64_t>(pool.size()));

    // Calibration windows, normalised like detection windows (windows that
    // fail the variance gate are left out): face patterns, and texture
    // windows cut at random from texture scenes at two scales, which is what
    // a detector scans.
    const int nCal = 1000, kNegCal = 8192;
    std::vector<uint8_t> px(static_cast<size_t>(nCal) * kWin * kWin);
    vj_synth_patches(mix64(seed ^ 0xCA11B8A7Eull), nCal, 0, px.data());
    std::vector<PatchII> pos, neg;
    for (int i = 0; i < nCal; ++i) {
        PatchII ii;
        patch_ii(px.data() + static_cast<size_t>(i) * kWin * kWin, &ii);
        if (ii.invNorm != 0.0f) pos.push_back(ii);
    }
    {
        const int tw[2] = {1280, 640}, th[2] = {720, 360};
        Rng crng(mix64(seed ^ 0x7E57u));
        uint8_t win[kWin * kWin];
        for (int t = 0; t < 2; ++t) {
            std::vector<uint8_t> tex(static_cast<size_t>(tw[t]) * th[t]);
            texture(mix64(seed + 0x1000u + static_cast<uint64_t>(t)), tw[t], th[t], tex.data(), tw[t]);
            for (int i = 0; i < kNegCal / 2; ++i) {
                const int x0 = crng.range(0, tw[t] - kWin), y0 = crng.range(0, th[t] - kWin);
                for (int y = 0; y < kWin; ++y)
                    std::memcpy(win + y * kWin, tex.data() + static_cast<size_t>(y0 + y) * tw[t] + x0, kWin);
                PatchII ii;
                patch_ii(win, &ii);
                if (ii.invNorm != 0.0f) neg.push_back(ii);
            }
        }
    }

    Rng rng(mix64(seed + 0x5CA5CADEull));
    std::vector<float> vals;
    std::vector<float> negSum(neg.size());
    std::vector<uint8_t> alive(neg.size(), 1);  // texture windows that passed every earlier stage
    int first = 0;
    for (int si = 0; si < stageCount; ++si) {
        std::fill(negSum.begin(), negSum.end(), 0.0f);
        for (int k = 0; k < sizes[static_cast<size_t>(si)]; ++k) {
            const int fi = static_cast<int>(rng.next() % pool.size());
            const vj_haar_feature& f = pool[static_cast<size_t>(fi)];
            vals.clear();
            for (const auto& ii : pos) vals.push_back(patch_response(f, ii));
            for (const auto& ii : neg) vals.push_back(patch_response(f, ii));
            std::vector<float> sorted(vals);
            std::sort(sorted.begin(), sorted.end());
            const size_t q = static_cast<size_t>(rng.range(300, 700)) * (sorted.size() - 1) / 1000;
            const float theta = 0.5f * (sorted[q] + sorted[std::min(q + 1, sorted.size() - 1)]);
            int posRight = 0, negRight = 0;
            for (size_t i = 0; i < pos.size(); ++i) posRight += vals[i] < theta ? 0 : 1;
            for (size_t i = 0; i < neg.size(); ++i) negRight += vals[pos.size() + i] < theta ? 0 : 1;
            const double fp = static_cast<double>(posRight) / static_cast<double>(pos.size());
            const double fn = static_cast<double>(negRight) / static_cast<double>(neg.size());
            const double sep = fp - fn;
            const float c = static_cast<float>(std::min(2.5, 0.2 + 4.0 * (sep < 0 ? -sep : sep)));
            const float left = sep >= 0 ? -c : c;
            const float right = sep >= 0 ? c : -c;
            vj_stump4& st = stumps[first + k];
            st.featureBits = bits_float(fi);
            st.theta = theta;
            st.leftVal = left;
            st.rightVal = right;
            for (size_t i = 0; i < neg.size(); ++i)
                negSum[i] += (vals[pos.size() + i] < theta) ? left : right;
        }
        // Threshold among the distinct stage sums whose rejection share
        // (sum < threshold) is closest to one half: over the texture windows
        // that reached this stage while at least 64 remain, else over all.
        std::vector<float> sortedSum;
        for (size_t i = 0; i < neg.size(); ++i)
            if (alive[i]) sortedSum.push_back(negSum[i]);
        if (sortedSum.size() < 64) sortedSum = negSum;
        std::sort(sortedSum.begin(), sortedSum.end());
        float thr = 0.0f;
        if (!sortedSum.empty()) {
            const double half = 0.5 * static_cast<double>(sortedSum.size());
            double bestGap = 1e300;
            for (size_t i = 0; i < sortedSum.size(); ++i) {
                if (i > 0 && sortedSum[i] == sortedSum[i - 1]) continue;
                const double gap = std::fabs(static_cast<double>(i) - half);
                if (gap < bestGap) {
                    bestGap = gap;
                    thr = sortedSum[i];
                }
            }
        }
        for (size_t i = 0; i < neg.size(); ++i)
            if (negSum[i] < thr) alive[i] = 0;
        stages[si].first = first;
        stages[si].ntrees = sizes[static_cast<size_t>(si)];
        stages[si].threshold = thr;
        first += sizes[static_cast<size_t>(si)];
    }
    return ok();
}

}  // extern "C"
