// mdg_insert.cpp -- seeded random sequential addition of spheres (host).
//
// The reference places DEM particles by rejection sampling against every
// placed sphere (insert.rs:523-571: uniform candidate in the region inset by
// the radius, reject if |d|_min-image < 1.1 (r_i + r_j)).  The acceptance rule
// is the same here; a uniform cell grid of side >= sep_factor * 2 rmax limits
// each test to the 27 surrounding cells.
#include <cmath>
#include <cstdint>
#include <vector>

#include "../../include/mdg.h"

namespace {

// xoshiro256** (Blackman & Vigna, 2018), seeded through splitmix64.
struct Rng {
    uint64_t s[4];
    static uint64_t splitmix(uint64_t& x) {
        uint64_t z = (x += 0x9e3779b97f4a7c15ull);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        return z ^ (z >> 31);
    }
    explicit Rng(uint64_t seed) {
        for (auto& v : s) v = splitmix(seed);
    }
    static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    uint64_t next() {
        const uint64_t r = rotl(s[1] * 5, 7) * 9, t = s[1] << 17;
        s[2] ^= s[0];
        s[3] ^= s[1];
        s[1] ^= s[2];
        s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return r;
    }
    double uniform() { return (double)(next() >> 11) * 0x1.0p-53; }  // [0, 1)
};

}  // namespace

extern "C" int mdg_rsa_spheres(size_t n, const double box_lo[3], const double box_hi[3], double rmin, double rmax,
                               double sep_factor, int inset, uint64_t seed, uint64_t max_attempts,
                               double* pos_out, double* rad_out, size_t* placed) {
    if (!box_lo || !box_hi || !pos_out || !rad_out || !placed) return MDG_ERR_ARG;
    *placed = 0;
    if (!(rmin > 0.0) || !(rmax >= rmin) || !(sep_factor > 0.0)) return MDG_ERR_ARG;
    double L[3], lo[3], hi[3], cell[3];
    int nc[3];
    const double reach = sep_factor * 2.0 * rmax;
    for (int d = 0; d < 3; d++) {
        L[d] = box_hi[d] - box_lo[d];
        if (!(L[d] > 0.0)) return MDG_ERR_ARG;
        lo[d] = box_lo[d] + (inset ? rmax : 0.0);
        hi[d] = box_hi[d] - (inset ? rmax : 0.0);
        if (!(hi[d] > lo[d])) return MDG_ERR_ARG;
        const double c = std::floor(L[d] / reach);
        nc[d] = c < 1.0 ? 1 : (c > 1024.0 ? 1024 : (int)c);
        cell[d] = L[d] / nc[d];
    }
    const size_t ncell = (size_t)nc[0] * nc[1] * nc[2];
    std::vector<int64_t> head(ncell, -1), next;
    next.reserve(n);
    // distinct neighbour-cell offsets per axis (fewer than 3 cells: no repeats)
    int off[3][3], noff[3];
    for (int d = 0; d < 3; d++) {
        noff[d] = nc[d] >= 3 ? 3 : nc[d];
        for (int k = 0; k < noff[d]; k++) off[d][k] = nc[d] >= 3 ? k - 1 : k;
    }
    const uint64_t limit = max_attempts ? max_attempts : (uint64_t)n * 20000ull;
    Rng rng(seed);
    size_t count = 0;
    const bool poly = rmax > rmin;
    auto cidx = [&](double x, int d) {
        int c = (int)std::floor((x - box_lo[d]) / cell[d]);
        c %= nc[d];
        return c < 0 ? c + nc[d] : c;
    };
    for (uint64_t att = 0; att < limit && count < n; att++) {
        double c[3];
        for (int d = 0; d < 3; d++) c[d] = lo[d] + (hi[d] - lo[d]) * rng.uniform();
        const double r = poly ? rmin + (rmax - rmin) * rng.uniform() : rmin;
        const int ci[3] = {cidx(c[0], 0), cidx(c[1], 1), cidx(c[2], 2)};
        bool ok = true;
        for (int a = 0; a < noff[0] && ok; a++)
            for (int b = 0; b < noff[1] && ok; b++)
                for (int e = 0; e < noff[2] && ok; e++) {
                    const int x = nc[0] >= 3 ? (ci[0] + off[0][a] + nc[0]) % nc[0] : off[0][a];
                    const int y = nc[1] >= 3 ? (ci[1] + off[1][b] + nc[1]) % nc[1] : off[1][b];
                    const int z = nc[2] >= 3 ? (ci[2] + off[2][e] + nc[2]) % nc[2] : off[2][e];
                    for (int64_t j = head[((size_t)x * nc[1] + y) * nc[2] + z]; j >= 0; j = next[j]) {
                        double r2 = 0.0;
                        for (int d = 0; d < 3; d++) {
                            double dx = pos_out[3 * j + d] - c[d];
                            dx -= L[d] * std::nearbyint(dx / L[d]);
                            r2 += dx * dx;
                        }
                        const double md = sep_factor * (r + rad_out[j]);
                        if (r2 <= md * md) {
                            ok = false;
                            break;
                        }
                    }
                }
        if (!ok) continue;
        for (int d = 0; d < 3; d++) pos_out[3 * count + d] = c[d];
        rad_out[count] = r;
        const size_t k = ((size_t)ci[0] * nc[1] + ci[1]) * nc[2] + ci[2];
        next.push_back(head[k]);
        head[k] = (int64_t)count;
        count++;
    }
    *placed = count;
    return count == n ? MDG_OK : MDG_ERR_ARG;
}
