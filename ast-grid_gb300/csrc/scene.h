// Scene definition for the octree smoke benchmark: split map, initial curl noise and the
// sphere source.  Header-only host C++ with no dependencies, so the same scene can be set up
// bit-identically by the library, by the CPU oracle and by the reference fixture harness.
//
// Frame: the reference solver is z-up (buoyancy acts on the MAC z faces,
// src/octree_omnigrid_solver3.cpp:932-940), so a y-up scene description maps y -> z.
//
// All arithmetic here is +, -, *, / on doubles (no libm calls), so with FP contraction
// disabled the results are identical on every IEEE-754 host.
#pragma once
#include <cstdint>
#include <cstring>
#include <vector>
#include <random>
#include <stdexcept>

namespace astg_scene {

struct Sphere {
    double cx, cy, cz, r;
};

// Default source: radius 0.06 at (0.5, 0.5, 0.12) in the z-up frame.
inline Sphere default_source() { return Sphere{0.5, 0.5, 0.12, 0.06}; }

inline bool inside(const Sphere& s, double x, double y, double z) {
    double dx = x - s.cx, dy = y - s.cy, dz = z - s.cz;
    // the reference tests (pos - c).norm() < r; compare squared distances instead of
    // calling sqrt, which is monotone and exact enough to give the same set except on
    // points at distance exactly r (none on these lattices).
    return dx * dx + dy * dy + dz * dz < s.r * s.r;
}

// Split map in the reference's convention (src/octree_layer3.cpp:20-23): one integer level id
// per finest cell, 0 = finest, levels-1 = coarsest; index = (z * res + y) * res + x.
//
// Rule: finest cells whose centre lies inside the source sphere (the cells that carry density
// above 0.01 at t=0) are marked, dilated by `buffer` cells (Chebyshev) at level 0; the result is
// coarsened to level 1 (a level-1 cell is refined when any child is marked), dilated by `buffer`
// cells at level 1, and so on.  Every refinement front is therefore surrounded by at least
// `buffer` cells of the next coarser level, which keeps the octree graded (ghost neighbours only
// ever differ by one level).
inline std::vector<int32_t> split_map(int res, int levels, const Sphere& src, int buffer = 2) {
    if (levels < 1 || res <= 0 || (res % (1 << (levels - 1))) != 0)
        throw std::runtime_error("split_map: resolution not divisible by 2^(levels-1)");
    const double dx = 1.0 / res;
    std::vector<int32_t> split((size_t)res * res * res, levels - 1);
    if (levels == 1) return split;
    // mark_k: cells of level k (resolution res>>k) that must be refined to level <= k
    std::vector<uint8_t> mark((size_t)res * res * res, 0);
    for (int z = 0; z < res; ++z)
        for (int y = 0; y < res; ++y)
            for (int x = 0; x < res; ++x)
                if (inside(src, (x + 0.5) * dx, (y + 0.5) * dx, (z + 0.5) * dx))
                    mark[((size_t)z * res + y) * res + x] = 1;
    int lres = res;
    for (int k = 0; k + 1 < levels; ++k) {
        // dilate mark at level k by `buffer`
        std::vector<uint8_t> dil((size_t)lres * lres * lres, 0);
        for (int z = 0; z < lres; ++z)
            for (int y = 0; y < lres; ++y)
                for (int x = 0; x < lres; ++x) {
                    if (!mark[((size_t)z * lres + y) * lres + x]) continue;
                    for (int dz = -buffer; dz <= buffer; ++dz)
                        for (int dy = -buffer; dy <= buffer; ++dy)
                            for (int dxx = -buffer; dxx <= buffer; ++dxx) {
                                int nx = x + dxx, ny = y + dy, nz = z + dz;
                                if (nx < 0 || ny < 0 || nz < 0 || nx >= lres || ny >= lres || nz >= lres) continue;
                                dil[((size_t)nz * lres + ny) * lres + nx] = 1;
                            }
                }
        // coarsen to level k+1: a parent is refined when any child is marked
        int cres = lres / 2;
        std::vector<uint8_t> par((size_t)cres * cres * cres, 0);
        for (int z = 0; z < lres; ++z)
            for (int y = 0; y < lres; ++y)
                for (int x = 0; x < lres; ++x)
                    if (dil[((size_t)z * lres + y) * lres + x])
                        par[((size_t)(z >> 1) * cres + (y >> 1)) * cres + (x >> 1)] = 1;
        // finest cells under a refined level-(k+1) parent that are not yet finer get level k
        for (int z = 0; z < res; ++z)
            for (int y = 0; y < res; ++y)
                for (int x = 0; x < res; ++x) {
                    int s = k + 1;
                    if (par[((size_t)(z >> s) * cres + (y >> s)) * cres + (x >> s)]) {
                        int32_t& v = split[((size_t)z * res + y) * res + x];
                        if (v > k) v = k;
                    }
                }
        mark.swap(par);
        lres = cres;
    }
    return split;
}

// Divergence-free curl noise u = amp * curl(A), A a trilinear interpolant of uniform random
// lattice values in [-1, 1) on a (K+1)^3 lattice over the unit cube, drawn from
// std::mt19937_64(seed) in the order (component, z, y, x).  The curl is evaluated exactly for
// the trilinear A inside the lattice cell that contains the point (cells clamped to [0, K-1]).
struct CurlNoise {
    int K;
    double amp, h, invh;
    std::vector<double> A[3];  // (K+1)^3 each, index (z*(K+1)+y)*(K+1)+x

    CurlNoise(uint64_t seed = 0, double amplitude = 1e-3, int lattice = 4)
        : K(lattice), amp(amplitude), h(1.0 / lattice), invh((double)lattice) {
        std::mt19937_64 rng(seed);
        const int n = (K + 1) * (K + 1) * (K + 1);
        for (int c = 0; c < 3; ++c) {
            A[c].resize(n);
            for (int i = 0; i < n; ++i) {
                // 53 random bits -> [0,1) exactly, then to [-1,1)
                double u = (double)(rng() >> 11) * (1.0 / 9007199254740992.0);
                A[c][i] = 2.0 * u - 1.0;
            }
        }
    }

    double at(int c, int x, int y, int z) const { return A[c][((size_t)z * (K + 1) + y) * (K + 1) + x]; }

    // gradient of component c of the trilinear interpolant at p
    void grad(int c, const double p[3], double g[3]) const {
        int i[3];
        double f[3];
        for (int a = 0; a < 3; ++a) {
            double r = p[a] * invh;
            int fi = (int)r;
            if (r < 0) fi = 0;
            if (fi > K - 1) fi = K - 1;
            if (fi < 0) fi = 0;
            i[a] = fi;
            double t = r - fi;
            f[a] = t < 0 ? 0 : (t > 1 ? 1 : t);
        }
        double v[2][2][2];
        for (int dz = 0; dz < 2; ++dz)
            for (int dy = 0; dy < 2; ++dy)
                for (int dx = 0; dx < 2; ++dx) v[dz][dy][dx] = at(c, i[0] + dx, i[1] + dy, i[2] + dz);
        // d/dx
        double gx = 0, gy = 0, gz = 0;
        for (int dz = 0; dz < 2; ++dz)
            for (int dy = 0; dy < 2; ++dy) {
                double wy = dy ? f[1] : 1.0 - f[1];
                double wz = dz ? f[2] : 1.0 - f[2];
                gx += (v[dz][dy][1] - v[dz][dy][0]) * (wy * wz);
            }
        for (int dz = 0; dz < 2; ++dz)
            for (int dx = 0; dx < 2; ++dx) {
                double wx = dx ? f[0] : 1.0 - f[0];
                double wz = dz ? f[2] : 1.0 - f[2];
                gy += (v[dz][1][dx] - v[dz][0][dx]) * (wx * wz);
            }
        for (int dy = 0; dy < 2; ++dy)
            for (int dx = 0; dx < 2; ++dx) {
                double wx = dx ? f[0] : 1.0 - f[0];
                double wy = dy ? f[1] : 1.0 - f[1];
                gz += (v[1][dy][dx] - v[0][dy][dx]) * (wx * wy);
            }
        g[0] = gx * invh;
        g[1] = gy * invh;
        g[2] = gz * invh;
    }

    // velocity vector at p
    void velocity(const double p[3], double u[3]) const {
        double g0[3], g1[3], g2[3];
        grad(0, p, g0);
        grad(1, p, g1);
        grad(2, p, g2);
        u[0] = amp * (g2[1] - g1[2]);
        u[1] = amp * (g0[2] - g2[0]);
        u[2] = amp * (g1[0] - g0[1]);
    }
};

}  // namespace astg_scene
