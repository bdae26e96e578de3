// Seeded procedural scenes for the triangle path.  The reference renders a
// compile-time list of 5 spheres (src/gpu/scene.glsl:4-11) and has no mesh
// or scene loading; these generators are new and produce the workloads the
// kernels are measured on:
//   heightfield + boxes     (64x64 grid, 8192 + 32*12 = 8576 triangles)
//   icosphere field         (200 icospheres, 4 subdivisions, Perlin-displaced,
//                            on a 10,240-triangle ground plane)
// Everything is computed in double and rounded to float once, so the output
// is the same on every host that has a correctly rounded libm sin/cos for
// the few trigonometric calls (the ULP-level exceptions only move vertices
// by one float ULP and are caught by the mesh-hash test).
#include "mrt_host.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <vector>

namespace {

constexpr double kPi = 3.14159265358979323846;

// SplitMix64 (Steele, Lea & Flood 2014): the seed stream of every generator.
struct Rng {
    uint64_t s;
    explicit Rng(uint64_t seed) : s(seed) {}
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return double(next() >> 11) * (1.0 / 9007199254740992.0); } // [0,1)
    double uniform(double a, double b) { return a + (b - a) * uniform(); }
};

struct D3 { double x, y, z; };
inline D3 sub(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline D3 add(D3 a, D3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline D3 mul(D3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline D3 cross(D3 a, D3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline double dot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline D3 normalize(D3 a) { double l = std::sqrt(dot(a, a)); return l > 0 ? mul(a, 1.0 / l) : D3{0, 0, 1}; }

uint32_t pack_albedo(Rng& rng) {
    // albedo U[0.2, 0.8] per channel, stored as UNORM8
    uint32_t r = uint32_t(std::lround(rng.uniform(0.2, 0.8) * 255.0));
    uint32_t g = uint32_t(std::lround(rng.uniform(0.2, 0.8) * 255.0));
    uint32_t b = uint32_t(std::lround(rng.uniform(0.2, 0.8) * 255.0));
    return r | (g << 8) | (b << 16) | (255u << 24);
}

struct MeshBuilder {
    std::vector<float> verts;
    std::vector<mrt_material> mats;
    void tri(D3 a, D3 b, D3 c, uint32_t albedo) {
        float fa[3] = {float(a.x), float(a.y), float(a.z)};
        float fb[3] = {float(b.x), float(b.y), float(b.z)};
        float fc[3] = {float(c.x), float(c.y), float(c.z)};
        verts.insert(verts.end(), fa, fa + 3);
        verts.insert(verts.end(), fb, fb + 3);
        verts.insert(verts.end(), fc, fc + 3);
        // geometric normal from the float vertices, in double
        D3 pa{fa[0], fa[1], fa[2]}, pb{fb[0], fb[1], fb[2]}, pc{fc[0], fc[1], fc[2]};
        D3 n = normalize(cross(sub(pb, pa), sub(pc, pa)));
        mrt_material m;
        m.normal[0] = float(n.x); m.normal[1] = float(n.y); m.normal[2] = float(n.z);
        m.albedo_rgba8 = albedo;
        mats.push_back(m);
    }
    int finish(mrt_mesh* out) {
        uint32_t n = uint32_t(mats.size());
        out->tri_count = n;
        out->pad = 0;
        out->verts = static_cast<float*>(std::malloc(sizeof(float) * 9 * std::max<size_t>(n, 1)));
        out->materials = static_cast<mrt_material*>(std::malloc(sizeof(mrt_material) * std::max<size_t>(n, 1)));
        if (!out->verts || !out->materials) {
            std::free(out->verts); std::free(out->materials);
            out->verts = nullptr; out->materials = nullptr;
            return MRT_ENOMEM;
        }
        std::memcpy(out->verts, verts.data(), sizeof(float) * verts.size());
        std::memcpy(out->materials, mats.data(), sizeof(mrt_material) * mats.size());
        float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (size_t i = 0; i < verts.size(); ++i) {
            lo[i % 3] = std::min(lo[i % 3], verts[i]);
            hi[i % 3] = std::max(hi[i % 3], verts[i]);
        }
        for (int a = 0; a < 3; ++a) { out->bounds_lo[a] = lo[a]; out->bounds_hi[a] = hi[a]; }
        return MRT_OK;
    }
};

void add_box(MeshBuilder& mb, D3 lo, D3 hi, uint32_t albedo) {
    D3 c[8];
    for (int i = 0; i < 8; ++i)
        c[i] = D3{(i & 1) ? hi.x : lo.x, (i & 2) ? hi.y : lo.y, (i & 4) ? hi.z : lo.z};
    // 6 faces, outward winding (counter-clockwise seen from outside)
    const int f[6][4] = {{0, 2, 3, 1}, {4, 5, 7, 6}, {0, 1, 5, 4}, {2, 6, 7, 3}, {0, 4, 6, 2}, {1, 3, 7, 5}};
    for (auto& q : f) {
        mb.tri(c[q[0]], c[q[1]], c[q[2]], albedo);
        mb.tri(c[q[0]], c[q[2]], c[q[3]], albedo);
    }
}

struct Heightfield {
    double amp[4], freq[4], cth[4], sth[4], phase[4];
    explicit Heightfield(Rng& rng, double extent) {
        for (int k = 0; k < 4; ++k) {
            double th = rng.uniform(0.0, 2.0 * kPi);
            cth[k] = std::cos(th);
            sth[k] = std::sin(th);
            phase[k] = rng.uniform(0.0, 2.0 * kPi);
            freq[k] = (2.0 * kPi / (0.5 * extent)) * std::ldexp(1.0, k) * rng.uniform(0.8, 1.2);
            amp[k] = 1.0 * std::ldexp(1.0, -k);
        }
    }
    double z(double x, double y) const {
        double s = 0.0;
        for (int k = 0; k < 4; ++k) s += amp[k] * std::sin(freq[k] * (x * cth[k] + y * sth[k]) + phase[k]);
        return s;
    }
};

void add_heightfield(MeshBuilder& mb, const Heightfield& hf, uint32_t grid, double x0, double y0,
                     double extent, uint32_t albedo) {
    const double cell = extent / grid;
    std::vector<D3> v((grid + 1) * (grid + 1));
    for (uint32_t j = 0; j <= grid; ++j)
        for (uint32_t i = 0; i <= grid; ++i) {
            double x = x0 + i * cell, y = y0 + j * cell;
            v[j * (grid + 1) + i] = D3{x, y, hf.z(x - x0 - 0.5 * extent, y - y0 - 0.5 * extent)};
        }
    for (uint32_t j = 0; j < grid; ++j)
        for (uint32_t i = 0; i < grid; ++i) {
            D3 a = v[j * (grid + 1) + i], b = v[j * (grid + 1) + i + 1];
            D3 c = v[(j + 1) * (grid + 1) + i + 1], d = v[(j + 1) * (grid + 1) + i];
            mb.tri(a, b, c, albedo);
            mb.tri(a, c, d, albedo);
        }
}

// Improved Perlin noise (Perlin, SIGGRAPH 2002): quintic fade, gradients
// from the 12 cube-edge directions, a seeded permutation table.
struct Perlin {
    int p[512];
    explicit Perlin(Rng& rng) {
        int perm[256];
        for (int i = 0; i < 256; ++i) perm[i] = i;
        for (int i = 255; i > 0; --i) {
            int j = int(rng.next() % uint64_t(i + 1));
            std::swap(perm[i], perm[j]);
        }
        for (int i = 0; i < 512; ++i) p[i] = perm[i & 255];
    }
    static double fade(double t) { return t * t * t * (t * (t * 6.0 - 15.0) + 10.0); }
    static double lerp(double t, double a, double b) { return a + t * (b - a); }
    static double grad(int h, double x, double y, double z) {
        int hh = h & 15;
        double u = hh < 8 ? x : y;
        double v = hh < 4 ? y : ((hh == 12 || hh == 14) ? x : z);
        return ((hh & 1) ? -u : u) + ((hh & 2) ? -v : v);
    }
    double noise(double x, double y, double z) const {
        double fx = std::floor(x), fy = std::floor(y), fz = std::floor(z);
        int X = int(fx) & 255, Y = int(fy) & 255, Z = int(fz) & 255;
        x -= fx; y -= fy; z -= fz;
        double u = fade(x), v = fade(y), w = fade(z);
        int A = p[X] + Y, AA = p[A] + Z, AB = p[A + 1] + Z;
        int B = p[X + 1] + Y, BA = p[B] + Z, BB = p[B + 1] + Z;
        return lerp(w,
                    lerp(v, lerp(u, grad(p[AA], x, y, z), grad(p[BA], x - 1, y, z)),
                         lerp(u, grad(p[AB], x, y - 1, z), grad(p[BB], x - 1, y - 1, z))),
                    lerp(v, lerp(u, grad(p[AA + 1], x, y, z - 1), grad(p[BA + 1], x - 1, y, z - 1)),
                         lerp(u, grad(p[AB + 1], x, y - 1, z - 1), grad(p[BB + 1], x - 1, y - 1, z - 1))));
    }
};

// Unit icosphere: the icosahedron with each face split into 4, `levels`
// times; midpoints are shared through an edge map so the mesh is closed.
void icosphere(uint32_t levels, std::vector<D3>& verts, std::vector<uint32_t>& faces) {
    const double t = (1.0 + std::sqrt(5.0)) / 2.0;
    verts = {{-1, t, 0}, {1, t, 0}, {-1, -t, 0}, {1, -t, 0}, {0, -1, t}, {0, 1, t},
             {0, -1, -t}, {0, 1, -t}, {t, 0, -1}, {t, 0, 1}, {-t, 0, -1}, {-t, 0, 1}};
    for (auto& v : verts) v = normalize(v);
    faces = {0, 11, 5, 0, 5, 1, 0, 1, 7, 0, 7, 10, 0, 10, 11, 1, 5, 9, 5, 11, 4, 11, 10, 2, 10, 7, 6,
             7, 1, 8, 3, 9, 4, 3, 4, 2, 3, 2, 6, 3, 6, 8, 3, 8, 9, 4, 9, 5, 2, 4, 11, 6, 2, 10, 8, 6, 7,
             9, 8, 1};
    for (uint32_t l = 0; l < levels; ++l) {
        std::map<uint64_t, uint32_t> mid;
        auto midpoint = [&](uint32_t a, uint32_t b) {
            uint64_t key = (uint64_t(std::min(a, b)) << 32) | std::max(a, b);
            auto it = mid.find(key);
            if (it != mid.end()) return it->second;
            uint32_t idx = uint32_t(verts.size());
            verts.push_back(normalize(mul(add(verts[a], verts[b]), 0.5)));
            mid.emplace(key, idx);
            return idx;
        };
        std::vector<uint32_t> nf;
        nf.reserve(faces.size() * 4);
        for (size_t f = 0; f < faces.size(); f += 3) {
            uint32_t a = faces[f], b = faces[f + 1], c = faces[f + 2];
            uint32_t ab = midpoint(a, b), bc = midpoint(b, c), ca = midpoint(c, a);
            uint32_t q[12] = {a, ab, ca, b, bc, ab, c, ca, bc, ab, bc, ca};
            nf.insert(nf.end(), q, q + 12);
        }
        faces.swap(nf);
    }
}

} // namespace

extern "C" {

void mrt_mesh_free(mrt_mesh* mesh) {
    if (!mesh) return;
    std::free(mesh->verts);
    std::free(mesh->materials);
    mesh->verts = nullptr;
    mesh->materials = nullptr;
    mesh->tri_count = 0;
}

int mrt_scene_heightfield_boxes(uint64_t seed, uint32_t grid, uint32_t boxes, mrt_mesh* out) {
    if (!out || grid == 0 || grid > 4096) return MRT_EINVAL;
    std::memset(out, 0, sizeof(*out));
    Rng rng(seed * 0x2545F4914F6CDD1Dull + 1);
    const double extent = 32.0;
    Heightfield hf(rng, extent);
    MeshBuilder mb;
    mb.verts.reserve(size_t(grid) * grid * 18 + size_t(boxes) * 108);
    uint32_t ground_albedo = pack_albedo(rng);
    add_heightfield(mb, hf, grid, -0.5 * extent, -0.5 * extent, extent, ground_albedo);
    for (uint32_t b = 0; b < boxes; ++b) {
        double sx = rng.uniform(0.5, 3.0), sy = rng.uniform(0.5, 3.0), sz = rng.uniform(0.5, 3.0);
        double cx = rng.uniform(-0.42 * extent, 0.42 * extent);
        double cy = rng.uniform(-0.42 * extent, 0.42 * extent);
        double base = hf.z(cx, cy) - 0.25;
        uint32_t albedo = pack_albedo(rng);
        add_box(mb, D3{cx - 0.5 * sx, cy - 0.5 * sy, base}, D3{cx + 0.5 * sx, cy + 0.5 * sy, base + sz}, albedo);
    }
    return mb.finish(out);
}

uint32_t mrt_heightfield_grid_for(uint32_t target_tris) {
    double g = std::sqrt(double(target_tris) / 2.0);
    return uint32_t(std::max(1.0, std::round(g)));
}

int mrt_scene_icospheres(uint64_t seed, uint32_t spheres, uint32_t levels, float rmin, float rmax,
                         uint32_t ground_tris, mrt_mesh* out) {
    if (!out || levels > 8 || !(rmin > 0.0f) || !(rmax >= rmin)) return MRT_EINVAL;
    std::memset(out, 0, sizeof(*out));
    Rng rng(seed * 0x9E3779B97F4A7C15ull + 7);
    Perlin perlin(rng);
    std::vector<D3> uv;
    std::vector<uint32_t> uf;
    icosphere(levels, uv, uf);

    // field of spheres over a square whose side grows with the count
    // (200 spheres: 90 x 90 units, about a fifth of the ground covered)
    const double half = 3.2 * std::sqrt(double(std::max<uint32_t>(spheres, 1)));
    MeshBuilder mb;
    mb.verts.reserve((size_t(spheres) * (uf.size() / 3) + ground_tris + 64) * 9);

    if (ground_tris > 0) {
        // gx * gy * 2 >= ground_tris with gy/gx = 5/4 (64 x 80 cells = 10,240)
        uint32_t gx = uint32_t(std::ceil(std::sqrt(ground_tris / 2.5)));
        uint32_t gy = uint32_t(std::ceil(double(ground_tris) / (2.0 * gx)));
        double ext = 6.0 * half;
        uint32_t albedo = pack_albedo(rng);
        for (uint32_t j = 0; j < gy; ++j)
            for (uint32_t i = 0; i < gx; ++i) {
                double x0 = -0.5 * ext + ext * i / gx, x1 = -0.5 * ext + ext * (i + 1) / gx;
                double y0 = -0.5 * ext + ext * j / gy, y1 = -0.5 * ext + ext * (j + 1) / gy;
                D3 a{x0, y0, 0}, b{x1, y0, 0}, c{x1, y1, 0}, d{x0, y1, 0};
                mb.tri(a, b, c, albedo);
                mb.tri(a, c, d, albedo);
            }
    }

    const double lr0 = std::log(double(rmin)), lr1 = std::log(double(rmax));
    std::vector<D3> pv(uv.size());
    for (uint32_t s = 0; s < spheres; ++s) {
        double r = std::exp(rng.uniform(lr0, lr1));
        double cx = rng.uniform(-half, half), cy = rng.uniform(-half, half);
        double cz = r * rng.uniform(0.9, 1.6);
        double nfreq = 2.0, ox = rng.uniform(0, 64), oy = rng.uniform(0, 64), oz = rng.uniform(0, 64);
        uint32_t albedo = pack_albedo(rng);
        for (size_t i = 0; i < uv.size(); ++i) {
            D3 n = uv[i];
            double disp = 0.05 * r * perlin.noise(n.x * nfreq + ox, n.y * nfreq + oy, n.z * nfreq + oz);
            pv[i] = add(D3{cx, cy, cz}, mul(n, r + disp));
        }
        for (size_t f = 0; f < uf.size(); f += 3) mb.tri(pv[uf[f]], pv[uf[f + 1]], pv[uf[f + 2]], albedo);
    }
    return mb.finish(out);
}

} // extern "C"
