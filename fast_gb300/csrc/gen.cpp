// Seeded synthetic microstructures: overlapping spheres and randomly oriented
// ellipsoids, 255 = solid and 0 = pore as the reference's generator writes
// them (fastlib/src/volume/VolumeGenerator.cpp:210-252, OCCUPIED = 255 at
// :218).  The reference's generator draws from an unseedable process-global
// std::default_random_engine (VolumeGenerator.cpp:14) and its packer needs an
// absent submodule, so these are the engine's own seeded stand-ins.
//
// Only +, -, *, / and sqrt are used (all correctly rounded in IEEE 754) and
// the file is compiled with -ffp-contract=off, so the same seed gives the same
// volume on x86-64 and aarch64 hosts.
#include <cmath>
#include <cstdint>
#include <cstring>

#include "fasttau.h"

namespace {

// xoshiro256** seeded through splitmix64 (public-domain generators by
// Blackman & Vigna).
struct Rng {
    uint64_t s[4];
    static uint64_t splitmix(uint64_t &x)
    {
        uint64_t z = (x += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    explicit Rng(uint64_t seed)
    {
        uint64_t x = seed;
        for (int i = 0; i < 4; i++) s[i] = splitmix(x);
    }
    static uint64_t rotl(uint64_t v, int k) { return (v << k) | (v >> (64 - k)); }
    uint64_t next()
    {
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
    // uniform in [0, 1) with 53 random bits
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    double uniform(double a, double b) { return a + (b - a) * uniform(); }
};

struct Vol {
    uint8_t *v;
    int64_t nx, ny, nz, N;
    int64_t solid = 0;
    void set(int64_t x, int64_t y, int64_t z)
    {
        uint8_t &c = v[x + nx * (y + ny * z)];
        if (c == 0) {
            c = 255;
            solid++;
        }
    }
};

int64_t clampi(int64_t v, int64_t lo, int64_t hi) { return v < lo ? lo : (v > hi ? hi : v); }

void add_sphere(Vol &V, double cx, double cy, double cz, double r)
{
    const double r2 = r * r;
    const int64_t x0 = clampi((int64_t)std::floor(cx - r), 0, V.nx - 1), x1 = clampi((int64_t)std::ceil(cx + r), 0, V.nx - 1);
    const int64_t y0 = clampi((int64_t)std::floor(cy - r), 0, V.ny - 1), y1 = clampi((int64_t)std::ceil(cy + r), 0, V.ny - 1);
    const int64_t z0 = clampi((int64_t)std::floor(cz - r), 0, V.nz - 1), z1 = clampi((int64_t)std::ceil(cz + r), 0, V.nz - 1);
    for (int64_t z = z0; z <= z1; z++) {
        const double dz = (double)z + 0.5 - cz;
        for (int64_t y = y0; y <= y1; y++) {
            const double dy = (double)y + 0.5 - cy;
            const double dyz = dy * dy + dz * dz;
            if (dyz > r2) continue;
            for (int64_t x = x0; x <= x1; x++) {
                const double dx = (double)x + 0.5 - cx;
                if (dx * dx + dyz <= r2) V.set(x, y, z);
            }
        }
    }
}

// Uniform random rotation: a uniform point on S^3 by rejection from the 4-cube,
// as a unit quaternion, turned into a rotation matrix.
void random_rotation(Rng &R, double M[3][3])
{
    double q[4], n2;
    do {
        for (int i = 0; i < 4; i++) q[i] = R.uniform(-1.0, 1.0);
        n2 = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
    } while (n2 > 1.0 || n2 < 1e-6);
    const double n = std::sqrt(n2);
    const double w = q[0] / n, x = q[1] / n, y = q[2] / n, z = q[3] / n;
    M[0][0] = 1 - 2 * (y * y + z * z); M[0][1] = 2 * (x * y - w * z);     M[0][2] = 2 * (x * z + w * y);
    M[1][0] = 2 * (x * y + w * z);     M[1][1] = 1 - 2 * (x * x + z * z); M[1][2] = 2 * (y * z - w * x);
    M[2][0] = 2 * (x * z - w * y);     M[2][1] = 2 * (y * z + w * x);     M[2][2] = 1 - 2 * (x * x + y * y);
}

void add_ellipsoid(Vol &V, double cx, double cy, double cz, const double M[3][3], double a, double b, double c)
{
    const double ia2 = 1.0 / (a * a), ib2 = 1.0 / (b * b), ic2 = 1.0 / (c * c);
    const double r = a > b ? (a > c ? a : c) : (b > c ? b : c);
    const int64_t x0 = clampi((int64_t)std::floor(cx - r), 0, V.nx - 1), x1 = clampi((int64_t)std::ceil(cx + r), 0, V.nx - 1);
    const int64_t y0 = clampi((int64_t)std::floor(cy - r), 0, V.ny - 1), y1 = clampi((int64_t)std::ceil(cy + r), 0, V.ny - 1);
    const int64_t z0 = clampi((int64_t)std::floor(cz - r), 0, V.nz - 1), z1 = clampi((int64_t)std::ceil(cz + r), 0, V.nz - 1);
    for (int64_t z = z0; z <= z1; z++) {
        const double dz = (double)z + 0.5 - cz;
        for (int64_t y = y0; y <= y1; y++) {
            const double dy = (double)y + 0.5 - cy;
            for (int64_t x = x0; x <= x1; x++) {
                const double dx = (double)x + 0.5 - cx;
                // body-frame coordinates u = M^T d
                const double u = M[0][0] * dx + M[1][0] * dy + M[2][0] * dz;
                const double v = M[0][1] * dx + M[1][1] * dy + M[2][1] * dz;
                const double w = M[0][2] * dx + M[1][2] * dy + M[2][2] * dz;
                if (u * u * ia2 + v * v * ib2 + w * w * ic2 <= 1.0) V.set(x, y, z);
            }
        }
    }
}

int check(uint8_t *out, int64_t nx, int64_t ny, int64_t nz, double frac)
{
    if (!out) return FAST_NO_HOST_DATA;
    if (nx <= 0 || ny <= 0 || nz <= 0) return FAST_BAD_ARG;
    if (!(frac >= 0.0 && frac < 1.0)) return FAST_BAD_ARG;
    return FAST_OK;
}

}  // namespace

extern "C" {

FAST_API int fast_gen_spheres(uint8_t *out, int64_t nx, int64_t ny, int64_t nz, uint64_t seed, double r_min,
                              double r_max, double solid_fraction)
{
    int st = check(out, nx, ny, nz, solid_fraction);
    if (st != FAST_OK) return st;
    if (!(r_min > 0.0) || !(r_max >= r_min)) return FAST_BAD_ARG;
    Vol V{out, nx, ny, nz, nx * ny * nz};
    std::memset(out, 0, (size_t)V.N);
    const int64_t target = (int64_t)std::ceil(solid_fraction * (double)V.N);
    Rng R(seed);
    int64_t guard = 0;
    while (V.solid < target && guard++ < (int64_t)1 << 40) {
        const double cx = R.uniform(0.0, (double)nx), cy = R.uniform(0.0, (double)ny), cz = R.uniform(0.0, (double)nz);
        const double r = (r_max > r_min) ? R.uniform(r_min, r_max) : r_min;
        add_sphere(V, cx, cy, cz, r);
    }
    return FAST_OK;
}

FAST_API int fast_gen_ellipsoids(uint8_t *out, int64_t nx, int64_t ny, int64_t nz, uint64_t seed, double semi_major,
                                 double aspect, double solid_fraction)
{
    int st = check(out, nx, ny, nz, solid_fraction);
    if (st != FAST_OK) return st;
    if (!(semi_major > 0.0) || !(aspect > 0.0 && aspect <= 1.0)) return FAST_BAD_ARG;
    Vol V{out, nx, ny, nz, nx * ny * nz};
    std::memset(out, 0, (size_t)V.N);
    const int64_t target = (int64_t)std::ceil(solid_fraction * (double)V.N);
    const double a = semi_major, b = semi_major * aspect;
    Rng R(seed);
    int64_t guard = 0;
    while (V.solid < target && guard++ < (int64_t)1 << 40) {
        const double cx = R.uniform(0.0, (double)nx), cy = R.uniform(0.0, (double)ny), cz = R.uniform(0.0, (double)nz);
        double M[3][3];
        random_rotation(R, M);
        add_ellipsoid(V, cx, cy, cz, M, a, b, b);
    }
    return FAST_OK;
}

}  // extern "C"
