// scene_gen.cpp - seeded random sequential placement of spheres for the synthetic workloads.
//
// The reference builds scenes from files and has no generator; this is an engine-side helper
// for the seeded synthetic scenes (a drum filled by random sequential placement, hopper
// fills).  Host code only, portable: a fixed xoshiro256** stream seeded by splitmix64 and
// plain IEEE double arithmetic (the file is compiled with -ffp-contract=off), so the same seed
// places the same spheres on x86_64 and aarch64.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

#include "../../include/vedo_gpu.h"

namespace {

struct Xoshiro {
    uint64_t s[4];
    explicit Xoshiro(uint64_t seed) {
        for (int k = 0; k < 4; ++k) {                   // splitmix64
            seed += 0x9e3779b97f4a7c15ull;
            uint64_t z = seed;
            z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
            z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
            s[k] = z ^ (z >> 31);
        }
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
    double uniform() { return (double)(next() >> 11) * 0x1.0p-53; }   // [0, 1)
};

}  // namespace

extern "C" int vedo_place_spheres(uint32_t n, const double* radii, const double lo[3], const double hi[3],
                                  double cyl_radius, uint64_t seed, uint32_t max_tries, double* out,
                                  uint32_t* placed) {
    if (!radii || !lo || !hi || !out || !placed) return VEDO_ERR_INVALID_ARGUMENT;
    *placed = 0;
    double rmax = 0.0;
    for (uint32_t i = 0; i < n; ++i) {
        if (!(radii[i] > 0.0)) return VEDO_ERR_INVALID_ARGUMENT;
        rmax = std::max(rmax, radii[i]);
    }
    for (int k = 0; k < 3; ++k)
        if (!(hi[k] > lo[k])) return VEDO_ERR_INVALID_ARGUMENT;
    const double h = 2.0 * rmax;
    uint64_t dims[3];
    uint64_t cells = 1;
    for (int k = 0; k < 3; ++k) {
        dims[k] = (uint64_t)std::floor((hi[k] - lo[k]) / h) + 1;
        cells *= dims[k];
    }
    if (cells > (1ull << 31)) return VEDO_ERR_INVALID_ARGUMENT;      // region far too large for the spheres
    std::vector<int32_t> head(cells, -1), next(n, -1);
    auto cell_of = [&](const double* p, int64_t c[3]) {
        for (int k = 0; k < 3; ++k) {
            int64_t v = (int64_t)std::floor((p[k] - lo[k]) / h);
            c[k] = v < 0 ? 0 : (v >= (int64_t)dims[k] ? (int64_t)dims[k] - 1 : v);
        }
    };
    Xoshiro rng(seed);
    uint32_t count = 0;
    for (uint32_t i = 0; i < n; ++i) {
        const double r = radii[i];
        double* p = out + 3 * (size_t)i;
        p[0] = p[1] = p[2] = std::numeric_limits<double>::quiet_NaN();
        bool room = true;
        for (int k = 0; k < 3; ++k) room = room && hi[k] - lo[k] > 2.0 * r;
        if (!room || (cyl_radius > 0.0 && !(cyl_radius > r))) continue;
        for (uint32_t t = 0; t < max_tries; ++t) {
            double q[3];
            for (int k = 0; k < 3; ++k) q[k] = lo[k] + r + rng.uniform() * (hi[k] - lo[k] - 2.0 * r);
            if (cyl_radius > 0.0) {
                const double rr = cyl_radius - r;
                if (q[1] * q[1] + q[2] * q[2] > rr * rr) continue;
            }
            int64_t c[3];
            cell_of(q, c);
            bool ok = true;
            for (int64_t dx = -1; dx <= 1 && ok; ++dx)
                for (int64_t dy = -1; dy <= 1 && ok; ++dy)
                    for (int64_t dz = -1; dz <= 1 && ok; ++dz) {
                        const int64_t x = c[0] + dx, y = c[1] + dy, z = c[2] + dz;
                        if (x < 0 || y < 0 || z < 0 || x >= (int64_t)dims[0] || y >= (int64_t)dims[1] ||
                            z >= (int64_t)dims[2])
                            continue;
                        for (int32_t o = head[((uint64_t)x * dims[1] + (uint64_t)y) * dims[2] + (uint64_t)z]; o >= 0;
                             o = next[o]) {
                            const double* s = out + 3 * (size_t)o;
                            const double ex = q[0] - s[0], ey = q[1] - s[1], ez = q[2] - s[2];
                            const double R = r + radii[o];
                            if (ex * ex + ey * ey + ez * ez < R * R) {
                                ok = false;
                                break;
                            }
                        }
                    }
            if (!ok) continue;
            std::memcpy(p, q, sizeof(q));
            const uint64_t ci = ((uint64_t)c[0] * dims[1] + (uint64_t)c[1]) * dims[2] + (uint64_t)c[2];
            next[i] = head[ci];
            head[ci] = (int32_t)i;
            ++count;
            break;
        }
    }
    *placed = count;
    return VEDO_OK;
}
