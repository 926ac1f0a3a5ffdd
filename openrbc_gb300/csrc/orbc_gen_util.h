// Helpers shared by the host-side workload generators (not part of the ABI).
#pragma once

#include <cmath>
#include <cstdint>
#include <vector>

namespace orbc_gen {

/* Counter-based stream: Philox4x32-10 (Salmon et al., SC'11) over a 64-bit
 * counter, four 32-bit words per call. */
struct Stream {
    uint32_t k0, k1;
    uint64_t ctr = 0;
    uint32_t buf[4];
    int left = 0;
    explicit Stream(uint64_t seed, uint32_t lane = 0) : k0(uint32_t(seed) ^ (lane * 0x85EBCA6Bu)), k1(uint32_t(seed >> 32) + lane) {}
    uint32_t next() {
        if (left == 0) {
            uint32_t c0 = uint32_t(ctr), c1 = uint32_t(ctr >> 32), c2 = 0x243F6A88u, c3 = 0x85A308D3u;
            uint32_t a = k0, b = k1;
            for (int r = 0; r < 10; ++r) {
                const uint64_t p0 = uint64_t(0xD2511F53u) * c0, p1 = uint64_t(0xCD9E8D57u) * c2;
                const uint32_t n0 = uint32_t(p1 >> 32) ^ c1 ^ a, n2 = uint32_t(p0 >> 32) ^ c3 ^ b;
                c1 = uint32_t(p1);
                c3 = uint32_t(p0);
                c0 = n0;
                c2 = n2;
                a += 0x9E3779B9u;
                b += 0xBB67AE85u;
            }
            buf[0] = c0;
            buf[1] = c1;
            buf[2] = c2;
            buf[3] = c3;
            ++ctr;
            left = 4;
        }
        return buf[4 - left--];
    }
    double u01() {  // (0, 1)
        const uint64_t hi = next() >> 5, lo = next() >> 6;
        return (double(hi * 67108864ull + lo) + 0.5) / 9007199254740992.0;
    }
    double gauss() {  // Box-Muller
        const double u = u01(), v = u01();
        return std::sqrt(-2.0 * std::log(u)) * std::cos(2.0 * M_PI * v);
    }
};

/* Spatial hash of points with cell size h (open addressing on cell keys). */
struct PointHash {
    double h;
    std::vector<int64_t> keys;
    std::vector<int> head;
    std::vector<int> next;
    std::vector<double> pts;
    size_t mask;
    PointHash(double cell, size_t expected) : h(cell) {
        size_t cap = 1024;
        while (cap < 2 * expected + 16) cap <<= 1;
        keys.assign(cap, INT64_MIN);
        head.assign(cap, -1);
        mask = cap - 1;
    }
    static int64_t key3(int64_t x, int64_t y, int64_t z) {
        return ((x + (1 << 20)) & 0x1FFFFF) | (((y + (1 << 20)) & 0x1FFFFF) << 21) | (((z + (1 << 20)) & 0x1FFFFF) << 42);
    }
    size_t slot(int64_t k) const {
        uint64_t x = uint64_t(k) * 0x9E3779B97F4A7C15ull;
        size_t s = size_t(x >> 20) & mask;
        while (keys[s] != INT64_MIN && keys[s] != k) s = (s + 1) & mask;
        return s;
    }
    void insert(const double *p) {
        const int id = int(next.size());
        pts.insert(pts.end(), p, p + 3);
        const int64_t k = key3(int64_t(std::floor(p[0] / h)), int64_t(std::floor(p[1] / h)), int64_t(std::floor(p[2] / h)));
        const size_t s = slot(k);
        keys[s] = k;
        next.push_back(head[s]);
        head[s] = id;
    }
    /* true if some stored point lies closer than r (r <= h) */
    bool near(const double *p, double r) const {
        const int64_t cx = int64_t(std::floor(p[0] / h)), cy = int64_t(std::floor(p[1] / h)), cz = int64_t(std::floor(p[2] / h));
        const double r2 = r * r;
        for (int dz = -1; dz <= 1; ++dz)
            for (int dy = -1; dy <= 1; ++dy)
                for (int dx = -1; dx <= 1; ++dx) {
                    const int64_t k = key3(cx + dx, cy + dy, cz + dz);
                    const size_t s = slot(k);
                    if (keys[s] != k) continue;
                    for (int id = head[s]; id >= 0; id = next[size_t(id)]) {
                        const double *q = &pts[3 * size_t(id)];
                        const double ex = p[0] - q[0], ey = p[1] - q[1], ez = p[2] - q[2];
                        if (ex * ex + ey * ey + ez * ez < r2) return true;
                    }
                }
        return false;
    }
};

inline void tilt_normal(Stream &rs, double tilt, double *n) {
    const double ang = tilt * rs.gauss();
    const double phi = 2.0 * M_PI * rs.u01();
    // axis (cos phi, sin phi, 0); rotating +z about it by ang
    n[0] = std::sin(ang) * std::sin(phi);
    n[1] = -std::sin(ang) * std::cos(phi);
    n[2] = std::cos(ang);
}

inline const double kMass[6] = {1, 4, 4, 1, 10, 10};

}  // namespace orbc_gen
