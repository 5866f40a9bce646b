// Host-side input preprocessing of the cloth builders (no device code):
// greedy constraint colouring and bend-pair extraction, the two steps of the
// reference's input pipeline whose Python loops dominate the cost of building
// large cloths (xpbd_core.py:730-747, 828-859).  Both follow the pipeline's
// rules exactly, so a cloth built with them is the same cloth.
#include <algorithm>
#include <cstdint>
#include <unordered_map>
#include <vector>

#include "xpbd_host.cuh"

#define XG_EXPORT extern "C" __attribute__((visibility("default")))

// Greedy first-fit colouring in constraint order: each pair takes the lowest
// colour used by neither endpoint so far (xpbd_core.py:828-859).  Endpoints
// outside [0, vertex_count) do not constrain.  Writes one colour per pair and
// returns the number of colours, or -1 on invalid arguments.
XG_EXPORT int xpbd_gb300_greedy_color(const int* pairs, int count, int vertex_count, int* colors) {
    if (count < 0 || vertex_count < 0 || (count > 0 && (!pairs || !colors))) return -1;
    // per vertex: a 64-colour mask, with an overflow list beyond 64 colours
    std::vector<uint64_t> used(vertex_count, 0ull);
    std::unordered_map<int, std::vector<int>> extra;
    int ncolors = 0;
    auto taken = [&](int v, int c) {
        if (v < 0 || v >= vertex_count) return false;
        if (c < 64) return ((used[v] >> c) & 1ull) != 0;
        auto it = extra.find(v);
        return it != extra.end() && std::find(it->second.begin(), it->second.end(), c) != it->second.end();
    };
    auto take = [&](int v, int c) {
        if (v < 0 || v >= vertex_count) return;
        if (c < 64)
            used[v] |= 1ull << c;
        else
            extra[v].push_back(c);
    };
    for (int k = 0; k < count; ++k) {
        const int a = pairs[2 * k], b = pairs[2 * k + 1];
        int c = 0;
        const uint64_t blocked = (a >= 0 && a < vertex_count ? used[a] : 0ull) | (b >= 0 && b < vertex_count ? used[b] : 0ull);
        if (~blocked != 0ull) {
            c = __builtin_ctzll(~blocked);
        } else {
            c = 64;
            while (taken(a, c) || taken(b, c)) ++c;
        }
        colors[k] = c;
        take(a, c);
        take(b, c);
        ncolors = std::max(ncolors, c + 1);
    }
    return ncolors;
}

// Bend pairs of a triangle mesh: for every edge, the vertex opposite it in
// the first triangle that has the edge is paired with the opposite vertex of
// every later triangle on the edge whose opposite vertex differs
// (xpbd_core.py:730-747).  Triangles are walked in order, their edges as
// (a, b), (b, c), (c, a).  Writes the distinct pairs (lower index first) in
// increasing order and returns their number, or -1 on invalid arguments or
// when more than `max_pairs` would be written.
XG_EXPORT int xpbd_gb300_bend_pairs(const int* triangles, int triangle_count, int* pairs, int max_pairs) {
    if (triangle_count < 0 || max_pairs < 0 || (triangle_count > 0 && !triangles)) return -1;
    std::unordered_map<uint64_t, int> first_opposite;
    first_opposite.reserve((size_t)triangle_count * 2);
    std::vector<uint64_t> found;
    for (int t = 0; t < triangle_count; ++t) {
        const int a = triangles[3 * t], b = triangles[3 * t + 1], c = triangles[3 * t + 2];
        const int edges[3][3] = {{a, b, c}, {b, c, a}, {c, a, b}};
        for (const auto& e : edges) {
            const int x = std::min(e[0], e[1]), y = std::max(e[0], e[1]), opp = e[2];
            const uint64_t key = ((uint64_t)(uint32_t)x << 32) | (uint32_t)y;
            auto it = first_opposite.find(key);
            if (it == first_opposite.end()) {
                first_opposite.emplace(key, opp);
            } else if (it->second != opp) {
                const int p = std::min(it->second, opp), q = std::max(it->second, opp);
                found.push_back(((uint64_t)(uint32_t)p << 32) | (uint32_t)q);
            }
        }
    }
    // order by (p, q) as signed ints, the order of sorted() on the pairs
    std::sort(found.begin(), found.end(), [](uint64_t u, uint64_t w) {
        const int up = (int)(uint32_t)(u >> 32), wp = (int)(uint32_t)(w >> 32);
        if (up != wp) return up < wp;
        return (int)(uint32_t)u < (int)(uint32_t)w;
    });
    found.erase(std::unique(found.begin(), found.end()), found.end());
    if ((long long)found.size() > (long long)max_pairs) return -1;
    for (size_t k = 0; k < found.size(); ++k) {
        pairs[2 * k] = (int)(uint32_t)(found[k] >> 32);
        pairs[2 * k + 1] = (int)(uint32_t)found[k];
    }
    return (int)found.size();
}
