// nbh_host.cpp — seeded universe generators and .universe file I/O (host code of libnbh).
//
// Generators implement the reference's UniverseGenerator shapes
// (src/ch/fhnw/woipv/nbody/simulation/universe/*.java) with a seeded xoshiro256** stream
// instead of Math.random(), so every universe can be reproduced from its seed.
// .universe files are the Java serialisation stream the reference reads and writes
// (universe/serialize/UniverseSerializer.java:25-34, SerializedUniverseGenerator.java:21-37).
#include "../../include/nbh.h"

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

namespace {

constexpr double kPi = 3.14159265358979323846;

struct Rng {
    uint64_t s[4];
    static uint64_t splitmix(uint64_t& x) {
        uint64_t z = (x += 0x9e3779b97f4a7c15ull);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        return z ^ (z >> 31);
    }
    explicit Rng(uint64_t seed) {
        uint64_t x = seed;
        for (auto& w : s) w = splitmix(x);
    }
    static uint64_t rotl(uint64_t v, int k) { return (v << k) | (v >> (64 - k)); }
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
    double uniform() { return (double)(next() >> 11) * 0x1.0p-53; }   // [0, 1)
    double normal() {                                                    // Box-Muller
        double u1 = uniform(), u2 = uniform();
        if (u1 < 1e-300) u1 = 1e-300;
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * kPi * u2);
    }
    void unit_ball(double& x, double& y, double& z) {   // rejection, as PlummerUniverseGenerator:20-25
        double sq;
        do {
            x = uniform() * 2.0 - 1.0;
            y = uniform() * 2.0 - 1.0;
            z = uniform() * 2.0 - 1.0;
            sq = x * x + y * y + z * z;
        } while (sq > 1.0 || sq == 0.0);
    }
    void direction(double& x, double& y, double& z) {
        unit_ball(x, y, z);
        const double s = 1.0 / std::sqrt(x * x + y * y + z * z);
        x *= s; y *= s; z *= s;
    }
};

bool bad(int32_t offset, int32_t n) { return offset < 0 || n < 1; }

// Plummer radius for a mass fraction u (inverse cumulative mass), scale radius a:
// r = a / sqrt(u^(-2/3) - 1) (PlummerUniverseGenerator.java:12).
double plummer_radius(double u, double a) {
    if (u <= 0.0) return 0.0;
    return a / std::sqrt(std::pow(u, -2.0 / 3.0) - 1.0);
}

// Speed fraction q of the escape speed by rejection from g(q) = q^2 (1-q^2)^3.5
// (Aarseth, Henon & Wielen 1974; PlummerUniverseGenerator.java:26-30).
double plummer_speed_fraction(Rng& g) {
    double q, y;
    do {
        q = g.uniform();
        y = g.uniform() * 0.1;
    } while (y > q * q * std::pow(1.0 - q * q, 3.5));
    return q;
}

int write_be32(FILE* f, uint32_t v) {
    unsigned char b[4] = {(unsigned char)(v >> 24), (unsigned char)(v >> 16), (unsigned char)(v >> 8),
                          (unsigned char)v};
    return fwrite(b, 1, 4, f) == 4 ? 0 : -1;
}

}  // namespace

extern "C" {

int nbh_generate_uniform_ball(uint64_t seed, int32_t offset, int32_t n, float radius, float vsigma, float* x,
                              float* y, float* z, float* vx, float* vy, float* vz, float* m) {
    if (bad(offset, n) || !x || !y || !z || !m || !(radius > 0.0f)) return NBH_ERR_INVALID;
    Rng g(seed);
    for (int i = 0; i < n; ++i) {
        double a, b, c;
        g.unit_ball(a, b, c);
        x[offset + i] = (float)(a * radius);
        y[offset + i] = (float)(b * radius);
        z[offset + i] = (float)(c * radius);
        m[offset + i] = 1.0f / (float)n;
    }
    for (int i = 0; i < n; ++i) {
        if (vx) vx[offset + i] = (float)(g.normal() * vsigma);
        if (vy) vy[offset + i] = (float)(g.normal() * vsigma);
        if (vz) vz[offset + i] = (float)(g.normal() * vsigma);
    }
    return NBH_OK;
}

int nbh_generate_plummer(uint64_t seed, int32_t offset, int32_t n, float a, float M, float* x, float* y, float* z,
                         float* vx, float* vy, float* vz, float* m) {
    if (bad(offset, n) || !x || !y || !z || !m || !(a > 0.0f) || !(M > 0.0f)) return NBH_ERR_INVALID;
    Rng g(seed);
    const double vscale = std::sqrt((double)M / (double)a);   // G = 1
    for (int i = 0; i < n; ++i) {
        const double r = plummer_radius(g.uniform() * 0.999, 1.0);   // mass fraction capped like :12
        double dx, dy, dz;
        g.direction(dx, dy, dz);
        x[offset + i] = (float)(dx * r * a);
        y[offset + i] = (float)(dy * r * a);
        z[offset + i] = (float)(dz * r * a);
        m[offset + i] = (float)((double)M / n);
        const double q = plummer_speed_fraction(g);
        const double v = q * std::sqrt(2.0 / std::sqrt(1.0 + r * r)) * vscale;   // :31
        g.direction(dx, dy, dz);
        if (vx) vx[offset + i] = (float)(dx * v);
        if (vy) vy[offset + i] = (float)(dy * v);
        if (vz) vz[offset + i] = (float)(dz * v);
    }
    return NBH_OK;
}

int nbh_generate_disc(uint64_t seed, int32_t offset, int32_t n, float rd, float zd, float mc, float halo_frac,
                      float* x, float* y, float* z, float* vx, float* vy, float* vz, float* m) {
    if (bad(offset, n) || n < 2 || !x || !y || !z || !m || !(rd > 0.0f) || !(zd > 0.0f) || !(mc >= 0.0f) ||
        !(halo_frac >= 0.0f && halo_frac < 1.0f))
        return NBH_ERR_INVALID;
    Rng g(seed);
    const int np = n - 1;                       // particles besides the central mass
    const int nh = (int)std::floor((double)halo_frac * np + 0.5);
    const int nd = np - nh;
    const double mp = 1.0 / np;                 // disc + halo hold unit mass
    const double Md = (double)nd * mp, Mh = (double)nh * mp;
    const double ah = 3.0 * rd;                 // halo scale radius
    auto enclosed = [&](double R) {             // spherical estimate of the mass inside R
        const double s = R / rd;
        const double disc = Md * (1.0 - (1.0 + s) * std::exp(-s));
        const double halo = Mh * R * R * R / std::pow(R * R + ah * ah, 1.5);
        return (double)mc + disc + halo;
    };
    // central point mass (RotatingDiskGalaxyGenerator.java:22 puts it at the first index)
    x[offset] = y[offset] = z[offset] = 0.0f;
    m[offset] = mc;
    if (vx) vx[offset] = 0.0f;
    if (vy) vy[offset] = 0.0f;
    if (vz) vz[offset] = 0.0f;
    for (int i = 1; i < n; ++i) {
        const int o = offset + i;
        m[o] = (float)mp;
        if (i <= nd) {
            // surface density ~ exp(-R/rd): R ~ Gamma(2, rd); vertical sech^2(z/zd) profile
            double u1 = g.uniform(), u2 = g.uniform();
            if (u1 < 1e-300) u1 = 1e-300;
            if (u2 < 1e-300) u2 = 1e-300;
            const double R = -rd * std::log(u1 * u2);
            const double phi = 2.0 * kPi * g.uniform();
            double uz = g.uniform();
            uz = std::fmin(std::fmax(uz, 1e-12), 1.0 - 1e-12);
            const double zz = zd * std::atanh(2.0 * uz - 1.0);
            const double cx = R * std::cos(phi), cy = R * std::sin(phi);
            x[o] = (float)cx;
            y[o] = (float)cy;
            z[o] = (float)zz;
            const double vc = R > 0.0 ? std::sqrt(enclosed(R) / R) : 0.0;   // near-circular orbit
            const double disp = 0.05 * vc;
            if (vx) vx[o] = (float)(-std::sin(phi) * vc + disp * g.normal());
            if (vy) vy[o] = (float)(std::cos(phi) * vc + disp * g.normal());
            if (vz) vz[o] = (float)(disp * g.normal());
        } else {
            const double r = plummer_radius(g.uniform() * 0.999, ah);
            double dx, dy, dz;
            g.direction(dx, dy, dz);
            x[o] = (float)(dx * r);
            y[o] = (float)(dy * r);
            z[o] = (float)(dz * r);
            const double vesc = std::sqrt(2.0 * enclosed(std::sqrt(r * r + ah * ah)) / std::sqrt(r * r + ah * ah));
            const double v = plummer_speed_fraction(g) * vesc;
            g.direction(dx, dy, dz);
            if (vx) vx[o] = (float)(dx * v);
            if (vy) vy[o] = (float)(dy * v);
            if (vz) vz[o] = (float)(dz * v);
        }
    }
    return NBH_OK;
}

int nbh_generate_random_cube(uint64_t seed, int32_t offset, int32_t n, float range, float* x, float* y, float* z,
                             float* m) {
    if (bad(offset, n) || !x || !y || !z || !m) return NBH_ERR_INVALID;
    Rng g(seed);
    for (int i = 0; i < n; ++i) {   // RandomCubicUniverseGenerator.java:14-17
        x[offset + i] = (float)((g.uniform() - 0.5) * range);
        y[offset + i] = (float)((g.uniform() - 0.5) * range);
        z[offset + i] = (float)((g.uniform() - 0.5) * range);
        m[offset + i] = 1.0f / (float)n;
    }
    return NBH_OK;
}

int nbh_generate_sphere_surface(uint64_t seed, int32_t offset, int32_t n, float* x, float* y, float* z, float* m) {
    if (bad(offset, n) || !x || !y || !z || !m) return NBH_ERR_INVALID;
    Rng g(seed);
    for (int i = 0; i < n; ++i) {   // SphericalUniverseGenerator.java:8-18
        const double omega = g.uniform() * 2.0 * kPi;
        const double u = g.uniform() * 2.0 - 1.0;
        const double s = std::sqrt(1.0 - u * u);
        x[offset + i] = (float)(s * std::cos(omega));
        y[offset + i] = (float)(s * std::sin(omega));
        z[offset + i] = (float)u;
        m[offset + i] = 1.0f / (float)n;
    }
    return NBH_OK;
}

int nbh_generate_fibonacci_sphere(uint64_t seed, int32_t offset, int32_t n, float* x, float* y, float* z, float* m) {
    if (bad(offset, n) || !x || !y || !z || !m) return NBH_ERR_INVALID;
    Rng g(seed);
    const double rnd = g.uniform() * n;   // MonteCarloSphericalUniverseGenerator.java:8-25
    const double o = 2.0 / (double)n;
    const double inc = kPi * (3.0 - std::sqrt(5.0));
    for (int i = 0; i < n; ++i) {
        const double yy = ((i * o) - 1.0) + (o / 2.0);
        const double r = std::sqrt(1.0 - yy * yy);
        const double phi = std::fmod(i + rnd, (double)n) * inc;
        x[offset + i] = (float)(std::cos(phi) * r);
        y[offset + i] = (float)yy;
        z[offset + i] = (float)(std::sin(phi) * r);
        m[offset + i] = 1.0f / (float)n;
    }
    return NBH_OK;
}

int nbh_generate_lonlat_sphere(uint64_t seed, int32_t offset, int32_t n, float* x, float* y, float* z, float* m) {
    if (bad(offset, n) || !x || !y || !z || !m) return NBH_ERR_INVALID;
    Rng g(seed);
    const double R = 5.0;   // LonLatSphericalUniverseGenerator.java:11-28
    for (int i = 0; i < n; ++i) {
        const double lon = g.uniform() * 2.0 * kPi;
        const double lat = g.uniform() * 2.0 * kPi;
        x[offset + i] = (float)(R * std::cos(lat) * std::cos(lon));
        y[offset + i] = (float)(R * std::cos(lat) * std::sin(lon));
        z[offset + i] = (float)(R * std::sin(lat));
        m[offset + i] = 1.0f / (float)n;
    }
    return NBH_OK;
}

int nbh_generate_rotating_disk(uint64_t seed, int32_t offset, int32_t n, float r, float vmul, float center_mass,
                               float* x, float* y, float* z, float* vx, float* vy, float* vz, float* m) {
    if (bad(offset, n) || !x || !y || !z || !m) return NBH_ERR_INVALID;
    Rng g(seed);
    const float kOffset = 0.05f;   // RotatingDiskGalaxyGenerator.java:5,17-41
    x[offset] = y[offset] = z[offset] = 0.0f;
    m[offset] = center_mass;
    if (vx) vx[offset] = 0.0f;
    if (vy) vy[offset] = 0.0f;
    if (vz) vz[offset] = 0.0f;
    for (int i = 1; i < n; ++i) {
        const int o = offset + i;
        const float rr = (float)(g.uniform() * r) + kOffset;
        const double alpha = g.uniform() * 2.0 * kPi;
        const float px = (float)(std::cos(alpha) * rr);
        const float py = (float)(std::sin(alpha) * rr);
        x[o] = px;
        y[o] = py;
        z[o] = (float)((g.uniform() - 0.5) / 8.0);
        m[o] = 1.0f / (float)n;
        const float v0 = (float)std::sqrt((m[offset] + m[o]) / (rr * rr * rr)) * vmul;
        if (vx) vx[o] = py * v0;
        if (vy) vy[o] = -px * v0;
        if (vz) vz[o] = 0.0f;
    }
    return NBH_OK;
}

// ---- .universe ----------------------------------------------------------------------
// ObjectOutputStream layout written by UniverseSerializer.java:25-34:
//   AC ED 00 05 | 77 04 <int n> | 75 72 00 02 '[' 'F' <8-byte serialVersionUID> 02 00 00 78 70
//   <int len> <len big-endian floats> | 6 x (75 71 00 7E 00 00 <int len> <floats>)

int nbh_universe_read(const char* path, int32_t* n_out, float* x, float* y, float* z, float* vx, float* vy, float* vz,
                      float* m) {
    if (!path || !n_out) return NBH_ERR_INVALID;
    FILE* f = std::fopen(path, "rb");
    if (!f) return NBH_ERR_INVALID;
    std::vector<unsigned char> d;
    unsigned char buf[1 << 16];
    size_t k;
    while ((k = std::fread(buf, 1, sizeof buf, f)) > 0) d.insert(d.end(), buf, buf + k);
    std::fclose(f);
    size_t pos = 0;
    auto need = [&](size_t c) { return pos + c <= d.size(); };
    auto be32 = [&]() {
        uint32_t v = ((uint32_t)d[pos] << 24) | ((uint32_t)d[pos + 1] << 16) | ((uint32_t)d[pos + 2] << 8) | d[pos + 3];
        pos += 4;
        return v;
    };
    if (!need(10) || d[0] != 0xAC || d[1] != 0xED || d[2] != 0x00 || d[3] != 0x05 || d[4] != 0x77 || d[5] != 0x04)
        return NBH_ERR_INVALID;   // the older Integer-object layout is not readable by the reference either
    pos = 6;
    const int32_t n = (int32_t)be32();
    if (n < 1) return NBH_ERR_INVALID;
    *n_out = n;
    if (!x) return NBH_OK;
    float* dst[7] = {x, y, z, vx, vy, vz, m};
    bool have_desc = false;
    for (int a = 0; a < 7; ++a) {
        if (!need(2) || d[pos] != 0x75) return NBH_ERR_INVALID;
        ++pos;
        if (d[pos] == 0x72) {   // class descriptor "[F"
            if (!need(19) || d[pos + 1] != 0x00 || d[pos + 2] != 0x02 || d[pos + 3] != '[' || d[pos + 4] != 'F')
                return NBH_ERR_INVALID;
            pos += 5 + 8;   // name + serialVersionUID
            if (d[pos] != 0x02 || d[pos + 1] != 0x00 || d[pos + 2] != 0x00 || d[pos + 3] != 0x78 || d[pos + 4] != 0x70)
                return NBH_ERR_INVALID;
            pos += 5;
            have_desc = true;
        } else if (d[pos] == 0x71 && have_desc) {   // back-reference to it
            if (!need(5)) return NBH_ERR_INVALID;
            pos += 5;
        } else {
            return NBH_ERR_INVALID;
        }
        if (!need(4)) return NBH_ERR_INVALID;
        const int32_t len = (int32_t)be32();
        if (len < n || !need((size_t)len * 4)) return NBH_ERR_INVALID;
        for (int i = 0; i < n; ++i) {
            const uint32_t v = be32();
            float fv;
            std::memcpy(&fv, &v, 4);
            if (dst[a]) dst[a][i] = fv;
        }
        pos += (size_t)(len - n) * 4;
    }
    return NBH_OK;
}

int nbh_universe_write(const char* path, int32_t n, const float* x, const float* y, const float* z, const float* vx,
                       const float* vy, const float* vz, const float* m) {
    if (!path || n < 1 || !x || !y || !z || !m) return NBH_ERR_INVALID;
    FILE* f = std::fopen(path, "wb");
    if (!f) return NBH_ERR_INVALID;
    static const unsigned char head[] = {0xAC, 0xED, 0x00, 0x05, 0x77, 0x04};
    static const unsigned char desc[] = {0x75, 0x72, 0x00, 0x02, '[',  'F',  0x0B, 0x9C, 0x81, 0x89,
                                         0x22, 0xE0, 0x0C, 0x42, 0x02, 0x00, 0x00, 0x78, 0x70};
    static const unsigned char ref[] = {0x75, 0x71, 0x00, 0x7E, 0x00, 0x00};
    int rc = 0;
    rc |= fwrite(head, 1, sizeof head, f) == sizeof head ? 0 : -1;
    rc |= write_be32(f, (uint32_t)n);
    const float* src[7] = {x, y, z, vx, vy, vz, m};
    std::vector<unsigned char> body((size_t)n * 4);
    for (int a = 0; a < 7; ++a) {
        if (a == 0) rc |= fwrite(desc, 1, sizeof desc, f) == sizeof desc ? 0 : -1;
        else rc |= fwrite(ref, 1, sizeof ref, f) == sizeof ref ? 0 : -1;
        rc |= write_be32(f, (uint32_t)n);
        for (int i = 0; i < n; ++i) {
            uint32_t v = 0;
            const float fv = src[a] ? src[a][i] : 0.0f;
            std::memcpy(&v, &fv, 4);
            body[4 * i] = (unsigned char)(v >> 24);
            body[4 * i + 1] = (unsigned char)(v >> 16);
            body[4 * i + 2] = (unsigned char)(v >> 8);
            body[4 * i + 3] = (unsigned char)v;
        }
        rc |= fwrite(body.data(), 1, body.size(), f) == body.size() ? 0 : -1;
    }
    rc |= std::fclose(f);
    return rc ? NBH_ERR_INVALID : NBH_OK;
}

}  // extern "C"
