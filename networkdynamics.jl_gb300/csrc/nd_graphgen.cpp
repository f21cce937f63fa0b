// Seeded random graph generators for the benchmark shapes (Watts–Strogatz,
// Barabási–Albert, random geometric).  Built as the host library libnd_graphgen.so.
//
// The reference builds its graphs with Graphs.jl (watts_strogatz, barabasi_albert) and
// enumerates edges with `edges(g)`, which for a SimpleGraph yields every undirected edge
// once as (src < dst) in lexicographic order.  The generators here return that order.
// They are not bit-identical to Graphs.jl's (different random streams); every consumer
// gets the graph from here, so GPU and CPU paths always share it.
//
// Randomness: splitmix64-seeded xoshiro256**; integer arithmetic and exactly
// representable doubles only, so x86-64 and aarch64 produce the same graphs.

#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <vector>

namespace {

struct Rng {
    uint64_t s[4];
    explicit Rng(uint64_t seed) {
        uint64_t x = seed;
        for (int i = 0; i < 4; ++i) {
            x += 0x9E3779B97F4A7C15ull;
            uint64_t z = x;
            z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
            z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
            s[i] = z ^ (z >> 31);
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
    double uniform() { return (double)(next() >> 11) * 0x1.0p-53; }  // [0, 1)
    uint64_t below(uint64_t n) {                                      // unbiased [0, n)
        uint64_t lim = UINT64_MAX - UINT64_MAX % n;
        uint64_t x;
        do x = next();
        while (x >= lim);
        return x % n;
    }
};

// Sort (a<b) pairs lexicographically and drop duplicates with a counting pass by source.
int64_t emit_sorted(int64_t n, std::vector<std::pair<int64_t, int64_t>>& pairs, int64_t* src, int64_t* dst,
                    int64_t cap) {
    std::vector<int64_t> cnt(n + 1, 0);
    for (auto& pr : pairs) {
        if (pr.first > pr.second) std::swap(pr.first, pr.second);
        cnt[pr.first + 1]++;
    }
    for (int64_t i = 0; i < n; ++i) cnt[i + 1] += cnt[i];
    std::vector<int64_t> col(pairs.size());
    std::vector<int64_t> pos(cnt.begin(), cnt.end() - 1);
    for (auto& pr : pairs) col[pos[pr.first]++] = pr.second;
    int64_t ne = 0;
    for (int64_t s = 0; s < n; ++s) {
        auto b = col.begin() + cnt[s], e = col.begin() + cnt[s + 1];
        std::sort(b, e);
        int64_t last = -1;
        for (auto it = b; it != e; ++it) {
            if (*it == last || *it == s) continue;  // duplicate or self loop
            last = *it;
            if (ne < cap) {
                src[ne] = s;
                dst[ne] = *it;
            }
            ++ne;
        }
    }
    return ne;
}

}  // namespace

extern "C" {

// Watts–Strogatz: ring lattice with k/2 neighbours on each side, each lattice edge's far
// end rewired with probability beta to a uniform vertex (no self loops, no duplicates).
// Returns the number of edges (written up to `cap`), or -1 on bad arguments.
int64_t nd_gen_watts_strogatz(int64_t n, int64_t k, double beta, uint64_t seed, int64_t* src, int64_t* dst,
                              int64_t cap) {
    if (n < 1 || k < 0 || k % 2 || k >= n || beta < 0 || beta > 1) return -1;
    Rng rng(seed);
    const int64_t half = k / 2;
    std::vector<std::vector<int64_t>> adj(n);
    auto has = [&](int64_t a, int64_t b) {
        const auto& l = adj[a];
        return std::find(l.begin(), l.end(), b) != l.end();
    };
    auto add = [&](int64_t a, int64_t b) {
        adj[a].push_back(b);
        adj[b].push_back(a);
    };
    auto del = [&](int64_t a, int64_t b) {
        auto& la = adj[a];
        la.erase(std::find(la.begin(), la.end(), b));
        auto& lb = adj[b];
        lb.erase(std::find(lb.begin(), lb.end(), a));
    };
    for (int64_t s = 1; s <= half; ++s)
        for (int64_t i = 0; i < n; ++i) add(i, (i + s) % n);
    for (int64_t s = 1; s <= half; ++s) {
        for (int64_t i = 0; i < n; ++i) {
            if (rng.uniform() >= beta) continue;
            const int64_t j = (i + s) % n;
            if (!has(i, j)) continue;
            if ((int64_t)adj[i].size() >= n - 1) continue;
            int64_t t;
            do t = (int64_t)rng.below((uint64_t)n);
            while (t == i || has(i, t));
            del(i, j);
            add(i, t);
        }
    }
    std::vector<std::pair<int64_t, int64_t>> pairs;
    pairs.reserve((size_t)(n * half));
    for (int64_t i = 0; i < n; ++i)
        for (int64_t j : adj[i])
            if (i < j) pairs.emplace_back(i, j);
    return emit_sorted(n, pairs, src, dst, cap);
}

// Barabási–Albert: m initial isolated vertices; every later vertex attaches m edges to
// distinct earlier vertices chosen with probability proportional to degree (the first
// new vertex attaches to all m initial ones).  ne = m (n - m).
int64_t nd_gen_barabasi_albert(int64_t n, int64_t m, uint64_t seed, int64_t* src, int64_t* dst, int64_t cap) {
    if (m < 1 || n <= m) return -1;
    Rng rng(seed);
    std::vector<int64_t> ends;  // every edge endpoint once: sampling from it is degree-proportional
    ends.reserve((size_t)(2 * m * (n - m)));
    std::vector<std::pair<int64_t, int64_t>> pairs;
    pairs.reserve((size_t)(m * (n - m)));
    std::vector<int64_t> chosen(m);
    for (int64_t v = m; v < n; ++v) {
        int64_t nc = 0;
        if (v == m) {
            for (int64_t t = 0; t < m; ++t) chosen[nc++] = t;
        } else {
            while (nc < m) {
                int64_t t = ends[rng.below(ends.size())];
                bool dup = false;
                for (int64_t q = 0; q < nc; ++q) dup |= chosen[q] == t;
                if (!dup) chosen[nc++] = t;
            }
        }
        for (int64_t q = 0; q < m; ++q) {
            pairs.emplace_back(chosen[q], v);
            ends.push_back(chosen[q]);
            ends.push_back(v);
        }
    }
    return emit_sorted(n, pairs, src, dst, cap);
}

// Random geometric graph in the unit square: n uniform points, an edge for every pair at
// distance < radius.  Positions are written to xy[2n] when xy is not NULL.
int64_t nd_gen_random_geometric(int64_t n, double radius, uint64_t seed, int64_t* src, int64_t* dst,
                                int64_t cap, double* xy) {
    if (n < 1 || !(radius > 0)) return -1;
    Rng rng(seed);
    std::vector<double> x(n), y(n);
    for (int64_t i = 0; i < n; ++i) {
        x[i] = rng.uniform();
        y[i] = rng.uniform();
        if (xy) {
            xy[2 * i] = x[i];
            xy[2 * i + 1] = y[i];
        }
    }
    const int64_t g = std::max<int64_t>(1, std::min<int64_t>((int64_t)(1.0 / radius), 4096));
    std::vector<int64_t> cell_cnt(g * g + 1, 0), cell_of(n);
    for (int64_t i = 0; i < n; ++i) {
        int64_t cx = std::min<int64_t>(g - 1, (int64_t)(x[i] * g));
        int64_t cy = std::min<int64_t>(g - 1, (int64_t)(y[i] * g));
        cell_of[i] = cy * g + cx;
        cell_cnt[cell_of[i] + 1]++;
    }
    for (int64_t c = 0; c < g * g; ++c) cell_cnt[c + 1] += cell_cnt[c];
    std::vector<int64_t> members(n), fill(cell_cnt.begin(), cell_cnt.end() - 1);
    for (int64_t i = 0; i < n; ++i) members[fill[cell_of[i]]++] = i;
    const double r2 = radius * radius;
    std::vector<std::pair<int64_t, int64_t>> pairs;
    for (int64_t i = 0; i < n; ++i) {
        const int64_t cx = cell_of[i] % g, cy = cell_of[i] / g;
        for (int64_t dy = -1; dy <= 1; ++dy)
            for (int64_t dx = -1; dx <= 1; ++dx) {
                const int64_t nx = cx + dx, ny = cy + dy;
                if (nx < 0 || ny < 0 || nx >= g || ny >= g) continue;
                const int64_t c = ny * g + nx;
                for (int64_t q = cell_cnt[c]; q < cell_cnt[c + 1]; ++q) {
                    const int64_t j = members[q];
                    if (j <= i) continue;
                    const double ddx = x[i] - x[j], ddy = y[i] - y[j];
                    const double d2 = ddx * ddx + ddy * ddy;
                    if (d2 < r2) pairs.emplace_back(i, j);
                }
            }
    }
    return emit_sorted(n, pairs, src, dst, cap);
}

}  // extern "C"
