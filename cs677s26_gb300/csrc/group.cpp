// Host post-processing of raw detections: canonical order and grouping.
//
// group_rectangles restates groupRectanglesCpu (face_vision_engine.cu:
// 1401-1539) step for step - the same x-sorted sweep, the same sequence of
// union-find unions (path compression, union by rank), the same cluster
// order - so its output equals the reference's on the same input list.  It
// only avoids work that cannot change the result: rectangles are swept from
// contiguous x-sorted arrays, a pair whose y distance exceeds the sweep reach
// is skipped before the full similarity test (the similarity delta never
// exceeds the reach), and the containment pass starts at the first cluster
// inside its x window instead of scanning from the left.
#include "group.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <thread>

namespace vjgb {
namespace {

// Stable counting sort of indices 0..n-1 by key[i] in [0, range).
void counting_order(const std::vector<int>& key, int range, std::vector<int>& order) {
    std::vector<int> cnt(static_cast<size_t>(range) + 1, 0);
    for (int k : key) ++cnt[static_cast<size_t>(k) + 1];
    for (int r = 0; r < range; ++r) cnt[static_cast<size_t>(r) + 1] += cnt[static_cast<size_t>(r)];
    order.resize(key.size());
    for (size_t i = 0; i < key.size(); ++i) order[static_cast<size_t>(cnt[static_cast<size_t>(key[i])]++)] = static_cast<int>(i);
}

// Indices sorted by (x, index).
void order_by_x(const std::vector<vj_detection>& v, std::vector<int>& order) {
    const int n = static_cast<int>(v.size());
    int lo = 0, hi = 0;
    for (int i = 0; i < n; ++i) {
        lo = i ? std::min(lo, v[i].x) : v[i].x;
        hi = i ? std::max(hi, v[i].x) : v[i].x;
    }
    if (n > 0 && static_cast<int64_t>(hi) - lo < (int64_t(1) << 22)) {
        std::vector<int> key(n);
        for (int i = 0; i < n; ++i) key[i] = v[i].x - lo;
        counting_order(key, hi - lo + 1, order);
        return;
    }
    order.resize(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&v](int a, int b) { return v[a].x < v[b].x; });
}

}  // namespace

void canonical_sort(std::vector<vj_detection>& v) {
    const size_t n = v.size();
    if (n < 2) return;
    std::vector<uint64_t> key(n), key2(n);
    std::vector<uint32_t> idx(n), idx2(n);
    uint64_t orAll = 0, andAll = ~uint64_t(0);
    for (size_t i = 0; i < n; ++i) {
        const uint64_t k = (static_cast<uint64_t>(static_cast<uint32_t>(v[i].scaleIdx)) << 32) |
                           (static_cast<uint64_t>(static_cast<uint16_t>(v[i].y)) << 16) |
                           static_cast<uint64_t>(static_cast<uint16_t>(v[i].x));
        key[i] = k;
        idx[i] = static_cast<uint32_t>(i);
        orAll |= k;
        andAll &= k;
    }
    const uint64_t varying = orAll ^ andAll;
    size_t cnt[257];
    for (int b = 0; b < 8; ++b) {
        const int sh = 8 * b;
        if (((varying >> sh) & 0xFFu) == 0) continue;  // digit equal in every key
        std::fill(cnt, cnt + 257, size_t(0));
        for (size_t i = 0; i < n; ++i) ++cnt[((key[i] >> sh) & 0xFFu) + 1];
        for (int d = 0; d < 256; ++d) cnt[d + 1] += cnt[d];
        for (size_t i = 0; i < n; ++i) {
            const size_t p = cnt[(key[i] >> sh) & 0xFFu]++;
            key2[p] = key[i];
            idx2[p] = idx[i];
        }
        key.swap(key2);
        idx.swap(idx2);
    }
    std::vector<vj_detection> out(n);
    for (size_t i = 0; i < n; ++i) out[i] = v[idx[i]];
    v.swap(out);
}

std::vector<vj_detection> group_rectangles(const std::vector<vj_detection>& in, int minNeighbors, float eps,
                                           int threads) {
    const int n = static_cast<int>(in.size());
    if (n == 0) return {};
    std::vector<int> parent(n), rnk(n, 0), order;
    for (int i = 0; i < n; ++i) parent[i] = i;
    auto find = [&](int x) {
        int r = x;
        while (parent[r] != r) r = parent[r];
        while (parent[x] != r) {
            const int nx = parent[x];
            parent[x] = r;
            x = nx;
        }
        return r;
    };
    auto unite = [&](int a, int b) {
        a = find(a);
        b = find(b);
        if (a == b) return;
        if (rnk[a] < rnk[b]) std::swap(a, b);
        parent[b] = a;
        if (rnk[a] == rnk[b]) ++rnk[a];
    };
    order_by_x(in, order);
    std::vector<int> sx(n), sy(n), sw(n), sh(n);
    for (int k = 0; k < n; ++k) {
        const vj_detection& d = in[order[k]];
        sx[k] = d.x;
        sy[k] = d.y;
        sw[k] = d.w;
        sh[k] = d.h;
    }
    // The similar pairs of sweep positions [o0, o1), in sweep order: the
    // (oi, oj) sequence whose unions the reference performs.
    auto sweep = [&](int o0, int o1, auto&& emit) {
        std::vector<int> cand;
        for (int oi = o0; oi < o1; ++oi) {
            const int ax = sx[oi], ay = sy[oi], aw = sw[oi], ah = sh[oi];
            const int reach = static_cast<int>(eps * static_cast<float>(aw + ah) * 0.5f);
            const int end = static_cast<int>(std::upper_bound(sx.begin() + oi + 1, sx.end(), ax + reach) - sx.begin());
            // Candidates in the x window whose y distance is within the reach
            // (|dy| <= delta <= reach is necessary): a bit mask per 64
            // rectangles, then the set bits in increasing order.
            cand.clear();
            const unsigned span = 2u * static_cast<unsigned>(reach);
            const int* yv = sy.data();
            for (int base = oi + 1; base < end; base += 64) {
                const int lim = std::min(64, end - base);
                uint64_t m = 0;
                for (int k = 0; k < lim; ++k)
                    m |= static_cast<uint64_t>(static_cast<unsigned>(yv[base + k] - ay + reach) <= span) << k;
                while (m) {
                    cand.push_back(base + __builtin_ctzll(m));
                    m &= m - 1;
                }
            }
            for (const int oj : cand) {
                const int bx = sx[oj];
                const int dy = ay - sy[oj];
                const int bw = sw[oj], bh = sh[oj];
                const int delta =
                    static_cast<int>(eps * static_cast<float>(std::min(aw, bw) + std::min(ah, bh)) * 0.5f);
                if (std::abs(ax - bx) <= delta && std::abs(dy) <= delta && std::abs(ax + aw - bx - bw) <= delta &&
                    std::abs(ay + ah - sy[oj] - bh) <= delta)
                    emit(order[oi], order[oj]);
            }
        }
    };
    const int T = (threads > 1 && n >= 4096) ? std::min(threads, 16) : 1;
    std::vector<std::vector<std::pair<int, int>>> pairs(static_cast<size_t>(T));
    if (T == 1) {
        sweep(0, n, unite);
    } else {
        std::vector<std::thread> th;
        for (int t = 0; t < T; ++t)
            th.emplace_back([&, t] {
                auto& part = pairs[static_cast<size_t>(t)];
                sweep(static_cast<int>(static_cast<int64_t>(n) * t / T),
                      static_cast<int>(static_cast<int64_t>(n) * (t + 1) / T),
                      [&part](int a, int b) { part.emplace_back(a, b); });
            });
        for (auto& x : th) x.join();
        for (const auto& part : pairs)
            for (const auto& pr : part) unite(pr.first, pr.second);
    }
    struct Acc {
        int64_t x = 0, y = 0, w = 0, h = 0;
        int count = 0;
        float best = -INFINITY;
        int scaleIdx = 0;
    };
    std::vector<Acc> acc(n);
    for (int i = 0; i < n; ++i) {
        Acc& c = acc[find(i)];
        c.x += in[i].x;
        c.y += in[i].y;
        c.w += in[i].w;
        c.h += in[i].h;
        c.count += 1;
        if (in[i].score > c.best) {
            c.best = in[i].score;
            c.scaleIdx = in[i].scaleIdx;
        }
    }
    std::vector<vj_detection> cl;
    std::vector<int> cc;
    const int minN = std::max(1, minNeighbors);
    for (int i = 0; i < n; ++i) {
        if (find(i) != i || acc[i].count <= minN) continue;
        const Acc& c = acc[i];
        vj_detection d;
        d.x = static_cast<int>(c.x / c.count);
        d.y = static_cast<int>(c.y / c.count);
        d.w = static_cast<int>(c.w / c.count);
        d.h = static_cast<int>(c.h / c.count);
        d.scaleIdx = c.scaleIdx;
        d.score = c.best;
        cl.push_back(d);
        cc.push_back(c.count);
    }
    int maxW = 0;
    for (const auto& d : cl) maxW = std::max(maxW, d.w);
    std::vector<int> co;
    order_by_x(cl, co);
    std::vector<int> cx(co.size());
    for (size_t k = 0; k < co.size(); ++k) cx[k] = cl[static_cast<size_t>(co[k])].x;
    std::vector<vj_detection> out;
    for (size_t i = 0; i < cl.size(); ++i) {
        const vj_detection& r1 = cl[i];
        const int n1 = cc[i];
        const float lb = static_cast<float>(r1.x + r1.w) - (1.0f + eps) * static_cast<float>(maxW);
        const float rb = static_cast<float>(r1.x) + eps * static_cast<float>(maxW);
        bool drop = false;
        const size_t k0 = static_cast<size_t>(std::lower_bound(cx.begin(), cx.end(), static_cast<int>(lb)) - cx.begin());
        for (size_t k = k0; k < co.size(); ++k) {
            const int o = co[k];
            const vj_detection& r2 = cl[static_cast<size_t>(o)];
            if (r2.x > static_cast<int>(rb)) break;
            if (static_cast<size_t>(o) == i) continue;
            const int n2 = cc[static_cast<size_t>(o)];
            const int dx = static_cast<int>(static_cast<float>(r2.w) * eps);
            const int dy = static_cast<int>(static_cast<float>(r2.h) * eps);
            if (r1.x >= r2.x - dx && r1.y >= r2.y - dy && r1.x + r1.w <= r2.x + r2.w + dx &&
                r1.y + r1.h <= r2.y + r2.h + dy && (n2 > std::max(3, n1) || n1 < 3)) {
                drop = true;
                break;
            }
        }
        if (!drop) out.push_back(r1);
    }
    return out;
}

}  // namespace vjgb
