// CPU ORACLE -- test infrastructure only.
//
// This file is the checker for the GB300 ray-tracing path, never part of
// the product: only tests/, __graft_entry__.smoke() and bench.py's
// cpu_baseline leg load it.  It is a scalar C++ restatement of MinoteRT's
// hot path plus the triangle/BVH parts that the reference lacks:
//
//   pcg / randomFloat / randomSpherePoint      src/gpu/random.glsl:10-31
//   raySphereIntersect / rayAt                 src/gpu/intersect.glsl:22-37
//   tracePrimaryRay + main (g-buffer)          src/gpu/primaryRay.comp:23-76
//   rotatedRandom / traceSecondaryRays / main  src/gpu/secondaryRays.comp:60-135
//   look / perspective / inverse / view        src/stx/math.ixx:739-861,
//                                              src/gfx/camera.ixx:26-44
//   watertight ray/triangle                    Woop, Benthin & Wald, JCGT 2013
//   quantised BVH8 decode + stack traversal    Ylitie, Karras & Laine, HPG 2017
//   directional-light path estimator           (new; specified in the design notes)
//
// Parity status: pinned to the reference's own shaders.  The reference ships
// no tests or golden vectors and its GPU path (GLSL through Vulkan) cannot
// run here, so its compute shaders are compiled for the host instead
// (oracle/glsl: a mechanical GLSL -> C++ rewrite of the sources where they
// lie, against a small model of GLSL's types and built-ins) and the tests
// compare this file with them: random.glsl, raySphereIntersect, the primary
// pass's g-buffer and the secondary pass's colour under the sky agree bit for
// bit (tests/test_oracle_glsl_pins.py, with vectors committed under
// tests/golden for machines without the reference tree).  The triangle /
// BVH8 / NEE parts have no counterpart in the reference; they are checked by
// analytic cases and brute-force cross-checks of the BVH traversal.
//
// FP32 mode reproduces the kernels' arithmetic order (explicit fma where the
// kernels use one, no contraction elsewhere; built with -ffp-contract=off),
// so primary hits and t are bit-identical.  FP64 mode evaluates the same
// estimator in double precision as the check of converged images.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <thread>
#include <vector>

namespace {

// ----------------------------------------------------------- data layouts
struct Node {  // 128 bytes, see include/mrt_cuda.h mrt_bvh8_node
    float origin[3];
    int8_t ex[3];
    uint8_t imask;
    uint32_t child_base, tri_base;
    uint8_t meta[8];
    uint8_t qlo[3][8];
    uint8_t qhi[3][8];
    uint32_t reserved[12];
};
static_assert(sizeof(Node) == 128, "node layout");
struct Tri {  // 48 bytes, BVH leaf order
    float v0[3]; uint32_t id;
    float v1[3]; uint32_t p1;
    float v2[3]; uint32_t p2;
};
static_assert(sizeof(Tri) == 48, "tri layout");
struct Mat { float n[3]; uint32_t albedo; };
struct Ray { float o[3]; float tmin; float d[3]; float tmax; };
struct Hit { uint32_t prim; float t; };
struct Consts {
    float view[16], proj[16], inv_view[16], inv_proj[16], prev_view[16];
    float cam_pos[3];
    uint32_t frame;
};
static_assert(sizeof(Consts) == 84 * 4, "consts layout");

constexpr uint32_t kMiss = 0xFFFFFFFFu;

// ----------------------------------------------------------------- random
uint32_t pcg(uint32_t& v) {
    uint32_t state = v * 747796405u + 2891336453u;
    uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    v = (word >> 22u) ^ word;
    return v;
}
float random_float(uint32_t& s) { return float(pcg(s) & 0xFFFFFFu) / 16777216.0f; }
float rotated_random(uint32_t& s, float rot) {
    float x = random_float(s) + rot;
    return x - std::floor(x);
}

// ------------------------------------------------------------ vec helpers
template <typename F> struct V3 { F x, y, z; };
template <typename F> V3<F> operator+(V3<F> a, V3<F> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <typename F> V3<F> operator-(V3<F> a, V3<F> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <typename F> V3<F> operator*(V3<F> a, F s) { return {a.x * s, a.y * s, a.z * s}; }
template <typename F> V3<F> cmul(V3<F> a, V3<F> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <typename F> F dot(V3<F> a, V3<F> b) { F r = a.x * b.x; r = r + a.y * b.y; r = r + a.z * b.z; return r; }
template <typename F> V3<F> normalize(V3<F> v) {
    F len = std::sqrt(dot(v, v));
    return {v.x / len, v.y / len, v.z / len};
}
template <typename F> F comp(V3<F> v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

// sin / cos / tan of a binary32 argument, evaluated in binary64 and rounded
// once: the same bits on every host (the C library's binary32 versions
// differ between x86-64 and AArch64 in the last place)
template <typename F> F sin_(F x) { return F(std::sin(double(x))); }
template <typename F> F cos_(F x) { return F(std::cos(double(x))); }
template <typename F> F tan_(F x) { return F(std::tan(double(x))); }

template <typename F> V3<F> sphere_point(F rx, F ry) {
    const F Pi = F(3.14159265359f);
    F ang1 = (rx + F(1)) * Pi;
    F u = ry;
    F s = std::sqrt(F(1) - u * u);
    return {s * cos_(ang1), s * sin_(ang1), u};
}

// column-major mat4 * vec4: sequential non-FMA dot per row (math.ixx:699)
void matvec(const float* m, float x, float y, float z, float w, float out[4]) {
    for (int r = 0; r < 4; ++r) {
        float acc = m[0 * 4 + r] * x;
        acc = acc + m[1 * 4 + r] * y;
        acc = acc + m[2 * 4 + r] * z;
        acc = acc + m[3 * 4 + r] * w;
        out[r] = acc;
    }
}
void matvec_d(const float* m, double x, double y, double z, double w, double out[4]) {
    for (int r = 0; r < 4; ++r)
        out[r] = double(m[r]) * x + double(m[4 + r]) * y + double(m[8 + r]) * z + double(m[12 + r]) * w;
}
void matmul(const float* l, const float* r, float* out) {
    for (int c = 0; c < 4; ++c)
        for (int row = 0; row < 4; ++row) {
            float acc = l[row] * r[c * 4 + 0];
            acc = acc + l[4 + row] * r[c * 4 + 1];
            acc = acc + l[8 + row] * r[c * 4 + 2];
            acc = acc + l[12 + row] * r[c * 4 + 3];
            out[c * 4 + row] = acc;
        }
}

// ------------------------------------------------------------- half float
uint16_t f2h(float f) {
    uint32_t x;
    std::memcpy(&x, &f, 4);
    uint32_t sign = (x >> 16) & 0x8000u;
    x &= 0x7FFFFFFFu;
    if (x >= 0x7F800000u) return uint16_t(sign | (x > 0x7F800000u ? 0x7E00u : 0x7C00u));
    if (x >= 0x477FF000u) return uint16_t(sign | 0x7C00u);
    if (x < 0x38800000u) {
        if (x < 0x33000000u) return uint16_t(sign);
        uint32_t e = x >> 23, m = (x & 0x7FFFFFu) | 0x800000u;
        uint32_t shift = 126u - e;
        uint32_t mh = m >> shift, rem = m & ((1u << shift) - 1u), half = 1u << (shift - 1u);
        if (rem > half || (rem == half && (mh & 1u))) mh++;
        return uint16_t(sign | mh);
    }
    uint32_t h = (x >> 13) - (112u << 10), rem = x & 0x1FFFu;
    if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) h++;
    return uint16_t(sign | h);
}
float h2f(uint16_t h) {
    uint32_t sign = uint32_t(h & 0x8000u) << 16, e = (h >> 10) & 0x1Fu, m = h & 0x3FFu, x;
    if (e == 0) {
        if (m == 0) x = sign;
        else {
            float f = float(m) * (1.0f / 16777216.0f);
            std::memcpy(&x, &f, 4);
            x |= sign;
        }
    } else if (e == 31) x = sign | 0x7F800000u | (m << 13);
    else x = sign | ((e + 112u) << 23) | (m << 13);
    float f;
    std::memcpy(&f, &x, 4);
    return f;
}

// ------------------------------------------------------- camera (FP32)
struct Cam { float pos[3], yaw, pitch, fov, znear; uint32_t w, h; };

void cam_view(const Cam& c, float* out) {
    // camera.ixx:19-35: direction from yaw/pitch, look(pos, dir, +Z)
    V3<float> dir{cos_(c.pitch) * cos_(c.yaw), cos_(c.pitch) * sin_(c.yaw), sin_(c.pitch)};
    V3<float> up{0.0f, 0.0f, 1.0f};
    auto cross = [](V3<float> l, V3<float> r) {
        return V3<float>{l.y * r.z - r.y * l.z, l.z * r.x - r.z * l.x, l.x * r.y - r.x * l.y};
    };
    auto dot0 = [](V3<float> a, V3<float> b) { float r = 0.0f; r += a.x * b.x; r += a.y * b.y; r += a.z * b.z; return r; };
    V3<float> s0 = cross(up, dir);
    float len = std::sqrt(dot0(s0, s0));
    V3<float> s{s0.x / len, s0.y / len, s0.z / len};
    V3<float> u = cross(dir, s);
    V3<float> p{c.pos[0], c.pos[1], c.pos[2]};
    for (int i = 0; i < 16; ++i) out[i] = (i % 5 == 0) ? 1.0f : 0.0f;
    // math.ixx:829-843, m[col*4 + row]
    out[0] = -s.x; out[4] = -s.y; out[8] = -s.z;
    out[1] = u.x;  out[5] = u.y;  out[9] = u.z;
    out[2] = dir.x; out[6] = dir.y; out[10] = dir.z;
    out[12] = dot0(s, p);
    out[13] = -dot0(u, p);
    out[14] = -dot0(dir, p);
}

void cam_proj(const Cam& c, float* out) {
    // math.ixx:848-861 with aspect = h / w (camera.ixx:38-41)
    float aspect = float(c.h) / float(c.w);
    float hh = 1.0f / tan_(0.5f * c.fov);
    float ww = hh * aspect;
    for (int i = 0; i < 16; ++i) out[i] = 0.0f;
    out[0] = ww;
    out[5] = hh;
    out[11] = 1.0f;
    out[14] = c.znear;
}

void inverse4(const float* m, float* out) {
    // math.ixx:761-818, written out term by term
    auto M = [&](int c, int r) { return m[c * 4 + r]; };
    float coef00 = M(2, 2) * M(3, 3) - M(3, 2) * M(2, 3);
    float coef02 = M(1, 2) * M(3, 3) - M(3, 2) * M(1, 3);
    float coef03 = M(1, 2) * M(2, 3) - M(2, 2) * M(1, 3);
    float coef04 = M(2, 1) * M(3, 3) - M(3, 1) * M(2, 3);
    float coef06 = M(1, 1) * M(3, 3) - M(3, 1) * M(1, 3);
    float coef07 = M(1, 1) * M(2, 3) - M(2, 1) * M(1, 3);
    float coef08 = M(2, 1) * M(3, 2) - M(3, 1) * M(2, 2);
    float coef10 = M(1, 1) * M(3, 2) - M(3, 1) * M(1, 2);
    float coef11 = M(1, 1) * M(2, 2) - M(2, 1) * M(1, 2);
    float coef12 = M(2, 0) * M(3, 3) - M(3, 0) * M(2, 3);
    float coef14 = M(1, 0) * M(3, 3) - M(3, 0) * M(1, 3);
    float coef15 = M(1, 0) * M(2, 3) - M(2, 0) * M(1, 3);
    float coef16 = M(2, 0) * M(3, 2) - M(3, 0) * M(2, 2);
    float coef18 = M(1, 0) * M(3, 2) - M(3, 0) * M(1, 2);
    float coef19 = M(1, 0) * M(2, 2) - M(2, 0) * M(1, 2);
    float coef20 = M(2, 0) * M(3, 1) - M(3, 0) * M(2, 1);
    float coef22 = M(1, 0) * M(3, 1) - M(3, 0) * M(1, 1);
    float coef23 = M(1, 0) * M(2, 1) - M(2, 0) * M(1, 1);
    float f0[4] = {coef00, coef00, coef02, coef03}, f1[4] = {coef04, coef04, coef06, coef07};
    float f2[4] = {coef08, coef08, coef10, coef11}, f3[4] = {coef12, coef12, coef14, coef15};
    float f4[4] = {coef16, coef16, coef18, coef19}, f5[4] = {coef20, coef20, coef22, coef23};
    float v0[4] = {M(1, 0), M(0, 0), M(0, 0), M(0, 0)}, v1[4] = {M(1, 1), M(0, 1), M(0, 1), M(0, 1)};
    float v2[4] = {M(1, 2), M(0, 2), M(0, 2), M(0, 2)}, v3[4] = {M(1, 3), M(0, 3), M(0, 3), M(0, 3)};
    float inv[4][4];
    const float sa[4] = {1, -1, 1, -1}, sb[4] = {-1, 1, -1, 1};
    for (int k = 0; k < 4; ++k) {
        inv[0][k] = ((v1[k] * f0[k] - v2[k] * f1[k]) + v3[k] * f2[k]) * sa[k];
        inv[1][k] = ((v0[k] * f0[k] - v2[k] * f3[k]) + v3[k] * f4[k]) * sb[k];
        inv[2][k] = ((v0[k] * f1[k] - v1[k] * f3[k]) + v3[k] * f5[k]) * sa[k];
        inv[3][k] = ((v0[k] * f2[k] - v1[k] * f4[k]) + v2[k] * f5[k]) * sb[k];
    }
    float d0 = M(0, 0) * inv[0][0], d1 = M(0, 1) * inv[1][0], d2 = M(0, 2) * inv[2][0], d3 = M(0, 3) * inv[3][0];
    float one_over = 1.0f / ((d0 + d1) + (d2 + d3));
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) out[c * 4 + r] = inv[c][r] * one_over;
}

// ---------------------------------------------------------- ray generation
struct FrameInfo {
    const Consts* c;
    uint32_t w, h;
    float pitch_x, pitch_y;
    float pv[16], ppv[16];
};

FrameInfo frame_info(const Consts* c, uint32_t w, uint32_t h) {
    FrameInfo f;
    f.c = c;
    f.w = w;
    f.h = h;
    f.pitch_x = 1.0f / float(w);
    f.pitch_y = 1.0f / float(h);
    matmul(c->proj, c->view, f.pv);
    matmul(c->proj, c->prev_view, f.ppv);
    return f;
}

// primaryRay.comp:46-51
void primary_ray(const FrameInfo& f, uint32_t x, uint32_t y, V3<float>& o, V3<float>& d) {
    float uvx = (float(x) + 0.5f) * f.pitch_x;
    float uvy = 1.0f - (float(y) + 0.5f) * f.pitch_y;
    float org[4], vd[4], wd[4];
    matvec(f.c->inv_view, 0.0f, 0.0f, 0.0f, 1.0f, org);
    matvec(f.c->inv_proj, uvx * 2.0f - 1.0f, uvy * 2.0f - 1.0f, 1.0f, 1.0f, vd);
    matvec(f.c->inv_view, vd[0], vd[1], vd[2], 0.0f, wd);
    o = {org[0], org[1], org[2]};
    d = normalize(V3<float>{wd[0], wd[1], wd[2]});
}
void primary_ray_d(const FrameInfo& f, uint32_t x, uint32_t y, V3<double>& o, V3<double>& d) {
    double uvx = (double(x) + 0.5) / double(f.w);
    double uvy = 1.0 - (double(y) + 0.5) / double(f.h);
    double org[4], vd[4], wd[4];
    matvec_d(f.c->inv_view, 0, 0, 0, 1, org);
    matvec_d(f.c->inv_proj, uvx * 2 - 1, uvy * 2 - 1, 1, 1, vd);
    matvec_d(f.c->inv_view, vd[0], vd[1], vd[2], 0, wd);
    o = {org[0], org[1], org[2]};
    d = normalize(V3<double>{wd[0], wd[1], wd[2]});
}

// ------------------------------------------------------------ ray/sphere
float ray_sphere(V3<float> o, V3<float> d, V3<float> c, float r) {
    V3<float> oc = o - c;
    float a = dot(d, d);
    float half_b = dot(oc, d);
    float cc = dot(oc, oc) - r * r;
    float disc = half_b * half_b - a * cc;
    if (disc < 0.0f) return -1.0f;
    return (-half_b - std::sqrt(disc)) / a;
}

// ------------------------------------------------- watertight ray/triangle
struct Pre32 {
    V3<float> o, d;
    float ix, iy, iz;
    uint32_t oct;
    int kx, ky, kz;
    float sx, sy, sz, okx, oky, okz;
};

float safe_inv(float d) {
    const float tiny = std::ldexp(1.0f, -80);
    float dd = std::fabs(d) < tiny ? std::copysign(tiny, d) : d;
    return 1.0f / dd;
}

Pre32 pre32(V3<float> o, V3<float> d) {
    Pre32 r;
    r.o = o;
    r.d = d;
    r.ix = safe_inv(d.x); r.iy = safe_inv(d.y); r.iz = safe_inv(d.z);
    r.oct = (r.ix < 0 ? 1u : 0u) | (r.iy < 0 ? 2u : 0u) | (r.iz < 0 ? 4u : 0u);
    float ax = std::fabs(d.x), ay = std::fabs(d.y), az = std::fabs(d.z);
    int kz = (ax >= ay && ax >= az) ? 0 : (ay >= az ? 1 : 2);
    int kx = (kz + 1) % 3, ky = (kx + 1) % 3;
    if (comp(d, kz) < 0.0f) std::swap(kx, ky);
    r.kx = kx; r.ky = ky; r.kz = kz;
    r.sx = comp(d, kx) / comp(d, kz);
    r.sy = comp(d, ky) / comp(d, kz);
    r.sz = 1.0f / comp(d, kz);
    r.okx = comp(o, kx); r.oky = comp(o, ky); r.okz = comp(o, kz);
    return r;
}

bool tri32(const Pre32& r, const float* a, const float* b, const float* c, float tmin, float& t_out) {
    float akx = a[r.kx] - r.okx, aky = a[r.ky] - r.oky, akz = a[r.kz] - r.okz;
    float bkx = b[r.kx] - r.okx, bky = b[r.ky] - r.oky, bkz = b[r.kz] - r.okz;
    float ckx = c[r.kx] - r.okx, cky = c[r.ky] - r.oky, ckz = c[r.kz] - r.okz;
    float Ax = std::fma(-r.sx, akz, akx), Ay = std::fma(-r.sy, akz, aky);
    float Bx = std::fma(-r.sx, bkz, bkx), By = std::fma(-r.sy, bkz, bky);
    float Cx = std::fma(-r.sx, ckz, ckx), Cy = std::fma(-r.sy, ckz, cky);
    float U = Cx * By - Cy * Bx;
    float V = Ax * Cy - Ay * Cx;
    float W = Bx * Ay - By * Ax;
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        U = float(double(Cx) * double(By) - double(Cy) * double(Bx));
        V = float(double(Ax) * double(Cy) - double(Ay) * double(Cx));
        W = float(double(Bx) * double(Ay) - double(By) * double(Ax));
    }
    if ((U < 0 || V < 0 || W < 0) && (U > 0 || V > 0 || W > 0)) return false;
    float det = (U + V) + W;
    if (det == 0.0f) return false;
    float Az = r.sz * akz, Bz = r.sz * bkz, Cz = r.sz * ckz;
    float T = std::fma(U, Az, std::fma(V, Bz, W * Cz));
    if (T == 0.0f || ((T < 0.0f) != (det < 0.0f))) return false;
    float t = T / det;
    if (!(t > tmin)) return false;
    t_out = t;
    return true;
}

// same test in double precision (shear + edge functions), long double
// recheck on exact zeros
bool tri64(V3<double> o, V3<double> d, const float* fa, const float* fb, const float* fc, double tmin, double& t_out) {
    double ax = std::fabs(d.x), ay = std::fabs(d.y), az = std::fabs(d.z);
    int kz = (ax >= ay && ax >= az) ? 0 : (ay >= az ? 1 : 2);
    int kx = (kz + 1) % 3, ky = (kx + 1) % 3;
    if (comp(d, kz) < 0.0) std::swap(kx, ky);
    double sx = comp(d, kx) / comp(d, kz), sy = comp(d, ky) / comp(d, kz), sz = 1.0 / comp(d, kz);
    double A[3] = {fa[0] - o.x, fa[1] - o.y, fa[2] - o.z};
    double B[3] = {fb[0] - o.x, fb[1] - o.y, fb[2] - o.z};
    double C[3] = {fc[0] - o.x, fc[1] - o.y, fc[2] - o.z};
    double Ax = A[kx] - sx * A[kz], Ay = A[ky] - sy * A[kz];
    double Bx = B[kx] - sx * B[kz], By = B[ky] - sy * B[kz];
    double Cx = C[kx] - sx * C[kz], Cy = C[ky] - sy * C[kz];
    double U = Cx * By - Cy * Bx, V = Ax * Cy - Ay * Cx, W = Bx * Ay - By * Ax;
    if (U == 0.0 || V == 0.0 || W == 0.0) {
        U = double((long double)Cx * By - (long double)Cy * Bx);
        V = double((long double)Ax * Cy - (long double)Ay * Cx);
        W = double((long double)Bx * Ay - (long double)By * Ax);
    }
    if ((U < 0 || V < 0 || W < 0) && (U > 0 || V > 0 || W > 0)) return false;
    double det = U + V + W;
    if (det == 0.0) return false;
    double T = U * sz * A[kz] + V * sz * B[kz] + W * sz * C[kz];
    double t = T / det;
    if (!(t > tmin)) return false;
    t_out = t;
    return true;
}

// ------------------------------------------------------ BVH8 traversal FP32
struct Counts { uint64_t nodes = 0, tris = 0; };

float b2f(uint8_t v) { return float(v); }

// Mirrors the kernels' traversal order (octant keys, lowest key first,
// push the rest of the group) and box arithmetic, so node and triangle
// counts are the ones the GPU sees.
void trace_bvh32(const Node* nodes, uint32_t nn, const Tri* tris, uint32_t nt, const Pre32& r, float tmin, float tmax,
                 bool any_hit, uint32_t& prim, float& thit, Counts* cnt, uint32_t* status) {
    float tbest = tmax;
    uint32_t best = kMiss;
    uint32_t g_base = 0, g_hits = 1u << r.oct, g_imask = 1u;
    struct E { uint32_t base, hits, imask; } stk[64];
    int sp = 0;
    const float robust = 1.0f + 1.0f / 1048576.0f;
    uint32_t iters = 0;
    bool done = false;
    while (!done) {
        if (g_hits == 0) {
            if (sp == 0) break;
            --sp;
            g_base = stk[sp].base; g_hits = stk[sp].hits; g_imask = stk[sp].imask;
        }
        uint32_t key = uint32_t(__builtin_ctz(g_hits));
        g_hits &= g_hits - 1u;
        uint32_t slot = key ^ r.oct;
        uint32_t node = g_base + uint32_t(__builtin_popcount(g_imask & ((1u << slot) - 1u)));
        if (g_hits) {
            if (sp >= 24) { if (status) *status |= 2u; break; }  // the kernels' 24-entry stack
            stk[sp++] = E{g_base, g_hits, g_imask};
        }
        if (++iters > nn + 64u) { if (status) *status |= 1u; break; }
        if (node >= nn) { if (status) *status |= 4u; break; }
        if (cnt) cnt->nodes++;
        const Node& N = nodes[node];
        float sc[3], ad[3];
        const float inv[3] = {r.ix, r.iy, r.iz};
        const float org[3] = {r.o.x, r.o.y, r.o.z};
        for (int a = 0; a < 3; ++a) {
            sc[a] = std::ldexp(1.0f, N.ex[a]) * inv[a];
            ad[a] = (N.origin[a] - org[a]) * inv[a];
        }
        uint32_t int_keys = 0, tri_mask = 0;
        for (int i = 0; i < 8; ++i) {
            float tn[3], tf[3];
            for (int a = 0; a < 3; ++a) {
                bool neg = inv[a] < 0.0f;
                float qn = b2f(neg ? N.qhi[a][i] : N.qlo[a][i]);
                float qf = b2f(neg ? N.qlo[a][i] : N.qhi[a][i]);
                tn[a] = std::fma(qn, sc[a], ad[a]);
                tf[a] = std::fma(qf, sc[a], ad[a]);
            }
            float tnear = std::fmax(std::fmax(tn[0], tn[1]), std::fmax(tn[2], tmin));
            float tfar = std::fmin(std::fmin(tf[0], tf[1]), std::fmin(tf[2], tbest));
            if (tnear <= tfar * robust) {
                uint32_t meta = N.meta[i];
                if ((N.imask >> i) & 1u) int_keys |= 1u << (uint32_t(i) ^ r.oct);
                else tri_mask |= (meta >> 5) << (meta & 31u);
            }
        }
        g_base = N.child_base;
        g_hits = int_keys;
        g_imask = N.imask;
        while (tri_mask) {
            uint32_t bit = uint32_t(__builtin_ctz(tri_mask));
            tri_mask &= tri_mask - 1u;
            uint32_t ti = N.tri_base + bit;
            if (ti >= nt) { if (status) *status |= 8u; done = true; break; }
            if (cnt) cnt->tris++;
            const Tri& T = tris[ti];
            float t;
            if (tri32(r, T.v0, T.v1, T.v2, tmin, t)) {
                if (any_hit) {
                    if (t < tmax) { best = T.id; tbest = t; done = true; break; }
                } else if (t < tbest || (t == tbest && T.id < best)) {
                    tbest = t;
                    best = T.id;
                }
            }
        }
    }
    prim = best;
    thit = best == kMiss ? tmax : tbest;
}

// FP64 traversal over the same BVH (visit order irrelevant; boxes in double)
void trace_bvh64(const Node* nodes, uint32_t nn, const Tri* tris, uint32_t nt, V3<double> o, V3<double> d, double tmin,
                 double tmax, bool any_hit, uint32_t& prim, double& thit) {
    double inv[3] = {1.0 / (d.x == 0 ? 1e-300 : d.x), 1.0 / (d.y == 0 ? 1e-300 : d.y), 1.0 / (d.z == 0 ? 1e-300 : d.z)};
    double org[3] = {o.x, o.y, o.z};
    double tbest = tmax;
    uint32_t best = kMiss;
    std::vector<uint32_t> stk;
    stk.reserve(128);
    stk.push_back(0);
    while (!stk.empty()) {
        uint32_t ni = stk.back();
        stk.pop_back();
        if (ni >= nn) continue;
        const Node& N = nodes[ni];
        uint32_t k_int = 0;
        for (int i = 0; i < 8; ++i) {
            if (N.meta[i] == 0) continue;
            bool internal = (N.imask >> i) & 1u;
            double tn = tmin, tf = tbest;
            for (int a = 0; a < 3; ++a) {
                double s = std::ldexp(1.0, N.ex[a]);
                double lo = double(N.origin[a]) + N.qlo[a][i] * s, hi = double(N.origin[a]) + N.qhi[a][i] * s;
                double t0 = (lo - org[a]) * inv[a], t1 = (hi - org[a]) * inv[a];
                if (t0 > t1) std::swap(t0, t1);
                tn = std::max(tn, t0);
                tf = std::min(tf, t1);
            }
            bool hit = tn <= tf * (1.0 + 1e-12) + 1e-300;
            if (internal) {
                uint32_t child = N.child_base + k_int;
                k_int++;
                if (hit) stk.push_back(child);
            } else if (hit) {
                uint32_t meta = N.meta[i];
                uint32_t cnt = uint32_t(__builtin_popcount(meta >> 5)), off = meta & 31u;
                for (uint32_t k = 0; k < cnt; ++k) {
                    uint32_t ti = N.tri_base + off + k;
                    if (ti >= nt) continue;
                    const Tri& T = tris[ti];
                    double t;
                    if (tri64(o, d, T.v0, T.v1, T.v2, tmin, t)) {
                        if (any_hit) {
                            if (t < tmax) { prim = T.id; thit = t; return; }
                        } else if (t < tbest || (t == tbest && T.id < best)) {
                            tbest = t;
                            best = T.id;
                        }
                    }
                }
            }
        }
    }
    prim = best;
    thit = best == kMiss ? tmax : tbest;
}

// ------------------------------------------------------------ path tracing
struct Scene {
    const Node* nodes; uint32_t nn;
    const Tri* tris; uint32_t nt;
    const Mat* mats; uint32_t nm;
    const float* spheres; uint32_t ns; // 8 floats each: c.xyz, r, albedo.xyz, pad
};

struct Params {
    uint32_t samples, max_bounces, rr_start, rng_mode, estimator, accumulate, frame_index, sort_rays;
    float sun[3], pad0, sun_e[3], pad1, sky[3], pad2;
};
static_assert(sizeof(Params) == 80, "params layout");

uint32_t initial_seed(uint32_t mode, uint32_t frame, uint32_t pixel) {
    uint32_t s = (frame << 1u) | 1u;
    if (mode == 1u) {
        uint32_t h = pixel * 0x9E3779B1u + s;
        s = pcg(h) | 1u;
    }
    return s;
}

float offset_axis(float p, float n) {
    const float kOrigin = 1.0f / 32.0f, kFloatScale = 1.0f / 65536.0f, kIntScale = 256.0f;
    int of = int(kIntScale * n);
    int32_t pb;
    std::memcpy(&pb, &p, 4);
    pb += (p < 0.0f ? -of : of);
    float pi;
    std::memcpy(&pi, &pb, 4);
    return std::fabs(p) < kOrigin ? std::fma(kFloatScale, n, p) : pi;
}
V3<float> offset_ray(V3<float> p, V3<float> n) { return {offset_axis(p.x, n.x), offset_axis(p.y, n.y), offset_axis(p.z, n.z)}; }

struct RayCounts { uint64_t primary = 0, ext = 0, shadow = 0; };

// One path (all samples) for pixel (x, y); F = float reproduces the
// kernels' order of operations, F = double is the FP64 judge.
extern "C" int orc_sky_escape(const float* dir, float* out);  // post.cpp

// Radiance of a path escaping along d: the bound atmosphere sky (post.cpp),
// else the constant sky.
inline V3<float> escape32(const V3<float>& sky, const V3<float>& d) {
    float dd[3] = {d.x, d.y, d.z}, o[3];
    if (orc_sky_escape(dd, o)) return V3<float>{o[0], o[1], o[2]};
    return sky;
}

template <typename F>
V3<F> shade_pixel(const Scene& sc, const FrameInfo& fi, const Params& p, const float* bn_rot, uint32_t bnw,
                  uint32_t bnh, uint32_t x, uint32_t y, uint32_t prim0, F t0, RayCounts& rc, uint32_t* status);

template <>
V3<float> shade_pixel<float>(const Scene& sc, const FrameInfo& fi, const Params& p, const float* bn_rot, uint32_t bnw,
                             uint32_t bnh, uint32_t x, uint32_t y, uint32_t prim0, float t0, RayCounts& rc,
                             uint32_t* status) {
    const uint32_t pix = y * fi.w + x;
    uint32_t rng = initial_seed(p.rng_mode, fi.c->frame, pix);
    const float rotx = bn_rot[2 * ((y % bnh) * bnw + (x % bnw))], roty = bn_rot[2 * ((y % bnh) * bnw + (x % bnw)) + 1];
    const V3<float> sky{p.sky[0], p.sky[1], p.sky[2]}, sun{p.sun[0], p.sun[1], p.sun[2]};
    const V3<float> sun_e{p.sun_e[0], p.sun_e[1], p.sun_e[2]};
    V3<float> L{0, 0, 0};
    V3<float> o0, d0;
    primary_ray(fi, x, y, o0, d0);
    for (uint32_t s = 0; s < p.samples; ++s) {
        if (prim0 == kMiss) { L = L + escape32(sky, d0); continue; }
        V3<float> beta{1, 1, 1};
        V3<float> o = o0, d = d0;
        uint32_t prim = prim0;
        float t = t0;
        for (uint32_t v = 0;; ++v) {
            V3<float> hp = o + d * t;
            const Mat& m = sc.mats[prim];
            V3<float> n{m.n[0], m.n[1], m.n[2]};
            if (dot(n, d) > 0.0f) n = V3<float>{-n.x, -n.y, -n.z};
            V3<float> rho{float(m.albedo & 0xFFu) / 255.0f, float((m.albedo >> 8) & 0xFFu) / 255.0f,
                          float((m.albedo >> 16) & 0xFFu) / 255.0f};
            if (p.estimator == 1u) {
                float cosl = dot(n, sun);
                if (cosl > 0.0f) {
                    V3<float> os = offset_ray(hp, n);
                    Pre32 sr = pre32(os, sun);
                    uint32_t sp;
                    float st;
                    trace_bvh32(sc.nodes, sc.nn, sc.tris, sc.nt, sr, 0.0f, INFINITY, true, sp, st, nullptr, status);
                    rc.shadow++;
                    if (sp == kMiss) {
                        float k = cosl * 0.318309886183790671538f;
                        L = L + cmul(cmul(beta, rho), sun_e) * k;
                    }
                }
            }
            beta = cmul(beta, rho);
            if (v >= p.max_bounces) break;
            float u1 = rotated_random(rng, rotx);
            float u2 = rotated_random(rng, roty);
            V3<float> spp = sphere_point<float>(u1 * 2.0f - 1.0f, u2 * 2.0f - 1.0f);
            V3<float> nd = n + spp;
            if (dot(nd, nd) == 0.0f) nd = n;
            nd = normalize(nd);
            if (p.rr_start != 0u && v + 1u > p.rr_start) {
                float q = std::fmax(std::fmax(beta.x, beta.y), beta.z);
                q = std::fmin(std::fmax(q, 0.05f), 1.0f);
                float u3 = rotated_random(rng, rotx);
                if (u3 >= q) break;
                beta = V3<float>{beta.x / q, beta.y / q, beta.z / q};
            }
            o = offset_ray(hp, n);
            d = nd;
            Pre32 er = pre32(o, d);
            trace_bvh32(sc.nodes, sc.nn, sc.tris, sc.nt, er, 0.0f, INFINITY, false, prim, t, nullptr, status);
            rc.ext++;
            if (prim == kMiss) { L = L + cmul(beta, escape32(sky, d)); break; }
        }
    }
    return L;
}

template <>
V3<double> shade_pixel<double>(const Scene& sc, const FrameInfo& fi, const Params& p, const float* bn_rot,
                               uint32_t bnw, uint32_t bnh, uint32_t x, uint32_t y, uint32_t prim0, double t0,
                               RayCounts& rc, uint32_t*) {
    const uint32_t pix = y * fi.w + x;
    uint32_t rng = initial_seed(p.rng_mode, fi.c->frame, pix);
    const float rotx = bn_rot[2 * ((y % bnh) * bnw + (x % bnw))], roty = bn_rot[2 * ((y % bnh) * bnw + (x % bnw)) + 1];
    const V3<double> sky{p.sky[0], p.sky[1], p.sky[2]}, sun{p.sun[0], p.sun[1], p.sun[2]};
    const V3<double> sun_e{p.sun_e[0], p.sun_e[1], p.sun_e[2]};
    V3<double> L{0, 0, 0};
    V3<double> o0, d0;
    primary_ray_d(fi, x, y, o0, d0);
    // the ray offset keeps the FP32 rule's magnitude (part of the estimator)
    auto offset_d = [](V3<double> hp, V3<double> n) {
        V3<float> hf{float(hp.x), float(hp.y), float(hp.z)}, nf{float(n.x), float(n.y), float(n.z)};
        V3<float> of = offset_ray(hf, nf);
        return V3<double>{hp.x + (double(of.x) - double(hf.x)), hp.y + (double(of.y) - double(hf.y)),
                          hp.z + (double(of.z) - double(hf.z))};
    };
    for (uint32_t s = 0; s < p.samples; ++s) {
        if (prim0 == kMiss) { L = L + sky; continue; }
        V3<double> beta{1, 1, 1};
        V3<double> o = o0, d = d0;
        uint32_t prim = prim0;
        double t = t0;
        for (uint32_t v = 0;; ++v) {
            V3<double> hp = o + d * t;
            const Mat& m = sc.mats[prim];
            V3<double> n{m.n[0], m.n[1], m.n[2]};
            if (dot(n, d) > 0.0) n = V3<double>{-n.x, -n.y, -n.z};
            V3<double> rho{double(m.albedo & 0xFFu) / 255.0, double((m.albedo >> 8) & 0xFFu) / 255.0,
                           double((m.albedo >> 16) & 0xFFu) / 255.0};
            if (p.estimator == 1u) {
                double cosl = dot(n, sun);
                if (cosl > 0.0) {
                    V3<double> os = offset_d(hp, n);
                    uint32_t sp;
                    double st;
                    trace_bvh64(sc.nodes, sc.nn, sc.tris, sc.nt, os, sun, 0.0, INFINITY, true, sp, st);
                    rc.shadow++;
                    if (sp == kMiss) L = L + cmul(cmul(beta, rho), sun_e) * (cosl / 3.14159265358979323846);
                }
            }
            beta = cmul(beta, rho);
            if (v >= p.max_bounces) break;
            double u1 = rotated_random(rng, rotx);
            double u2 = rotated_random(rng, roty);
            V3<double> spp = sphere_point<double>(u1 * 2.0 - 1.0, u2 * 2.0 - 1.0);
            V3<double> nd = n + spp;
            if (dot(nd, nd) == 0.0) nd = n;
            nd = normalize(nd);
            if (p.rr_start != 0u && v + 1u > p.rr_start) {
                double q = std::max(std::max(beta.x, beta.y), beta.z);
                q = std::min(std::max(q, 0.05), 1.0);
                double u3 = rotated_random(rng, rotx);
                if (u3 >= q) break;
                beta = beta * (1.0 / q);
            }
            o = offset_d(hp, n);
            d = nd;
            trace_bvh64(sc.nodes, sc.nn, sc.tris, sc.nt, o, d, 0.0, INFINITY, false, prim, t);
            rc.ext++;
            if (prim == kMiss) { L = L + cmul(beta, sky); break; }
        }
    }
    return L;
}

template <typename Fn> void parallel_rows(uint32_t rows, int threads, Fn fn) {
    if (threads <= 0) threads = int(std::max(1u, std::thread::hardware_concurrency()));
    std::atomic<uint32_t> next{0};
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t)
        pool.emplace_back([&, t] {
            for (;;) {
                uint32_t r = next.fetch_add(1);
                if (r >= rows) break;
                fn(r, t);
            }
        });
    for (auto& th : pool) th.join();
}

} // namespace

extern "C" {

uint32_t orc_pcg(uint32_t v) { return pcg(v); }
float orc_random_float(uint32_t* state) { return random_float(*state); }
float orc_rotated_random(uint32_t* state, float rot) { return rotated_random(*state, rot); }
void orc_random_sphere_point(float rx, float ry, float* out) {
    V3<float> p = sphere_point<float>(rx, ry);
    out[0] = p.x; out[1] = p.y; out[2] = p.z;
}
uint16_t orc_f2h(float f) { return f2h(f); }
float orc_h2f(uint16_t h) { return h2f(h); }
float orc_ray_sphere(const float* o, const float* d, const float* c, float r) {
    return ray_sphere({o[0], o[1], o[2]}, {d[0], d[1], d[2]}, {c[0], c[1], c[2]}, r);
}

// camera: pos[3], yaw, pitch, fov, near, w, h -> Consts (84 floats)
void orc_camera_consts(const float* pos, float yaw, float pitch, float fov, float znear, uint32_t w, uint32_t h,
                       const float* prev_pos, float prev_yaw, float prev_pitch, uint32_t frame, float* out) {
    Consts c;
    std::memset(&c, 0, sizeof(c));
    Cam cam{{pos[0], pos[1], pos[2]}, yaw, pitch, fov, znear, w, h};
    Cam prev{{prev_pos[0], prev_pos[1], prev_pos[2]}, prev_yaw, prev_pitch, fov, znear, w, h};
    cam_view(cam, c.view);
    cam_proj(cam, c.proj);
    inverse4(c.view, c.inv_view);
    inverse4(c.proj, c.inv_proj);
    cam_view(prev, c.prev_view);
    c.cam_pos[0] = pos[0]; c.cam_pos[1] = pos[1]; c.cam_pos[2] = pos[2];
    c.frame = frame;
    std::memcpy(out, &c, sizeof(c));
}

void orc_inverse4(const float* m, float* out) { inverse4(m, out); }

// Watertight test of one ray against one triangle; returns 1 on a hit.
int orc_intersect_tri(const float* o, const float* d, const float* v0, const float* v1, const float* v2, float tmin,
                      float* t) {
    Pre32 r = pre32({o[0], o[1], o[2]}, {d[0], d[1], d[2]});
    float tt;
    if (!tri32(r, v0, v1, v2, tmin, tt)) return 0;
    *t = tt;
    return 1;
}
int orc_intersect_tri64(const double* o, const double* d, const float* v0, const float* v1, const float* v2,
                        double tmin, double* t) {
    double tt;
    if (!tri64({o[0], o[1], o[2]}, {d[0], d[1], d[2]}, v0, v1, v2, tmin, tt)) return 0;
    *t = tt;
    return 1;
}

// Brute-force closest (or any) hit over original-order triangles.
void orc_trace_brute(const float* verts, uint32_t ntris, const Ray* rays, uint32_t n, Hit* hits, int any_hit,
                     int threads) {
    parallel_rows(n, threads, [&](uint32_t i, int) {
        const Ray& ry = rays[i];
        Pre32 r = pre32({ry.o[0], ry.o[1], ry.o[2]}, {ry.d[0], ry.d[1], ry.d[2]});
        float tb = ry.tmax;
        uint32_t best = kMiss;
        for (uint32_t k = 0; k < ntris; ++k) {
            float t;
            const float* v = verts + 9ull * k;
            if (tri32(r, v, v + 3, v + 6, ry.tmin, t)) {
                if (any_hit) {
                    if (t < ry.tmax) { best = k; tb = t; break; }
                } else if (t < tb || (t == tb && k < best)) {
                    tb = t;
                    best = k;
                }
            }
        }
        hits[i] = Hit{best, best == kMiss ? ry.tmax : tb};
    });
}

// BVH8 closest/any hit in FP32 (the kernels' order and arithmetic) with
// per-ray node/triangle counters (either may be NULL).
uint32_t orc_trace_bvh8(const Node* nodes, uint32_t nn, const Tri* tris, uint32_t nt, const Ray* rays, uint32_t n,
                        Hit* hits, int any_hit, uint32_t* nodes_v, uint32_t* tris_v, int threads) {
    std::atomic<uint32_t> status{0};
    parallel_rows(n, threads, [&](uint32_t i, int) {
        const Ray& ry = rays[i];
        Pre32 r = pre32({ry.o[0], ry.o[1], ry.o[2]}, {ry.d[0], ry.d[1], ry.d[2]});
        Counts c;
        uint32_t st = 0, prim;
        float t;
        trace_bvh32(nodes, nn, tris, nt, r, ry.tmin, ry.tmax, any_hit != 0, prim, t, &c, &st);
        hits[i] = Hit{prim, t};
        if (nodes_v) nodes_v[i] = uint32_t(c.nodes);
        if (tris_v) tris_v[i] = uint32_t(c.tris);
        if (st) status.fetch_or(st);
    });
    return status.load();
}

// BVH8 structural check: every original triangle referenced exactly once,
// child boxes (dequantised) contain their subtree's geometry, depth.
// info[0] = depth, info[1] = max triangles per node, info[2] = error code
// (0 ok, 1 bad index, 2 box not conservative, 3 triangle count mismatch,
//  4 triangle data mismatch, 5 bad meta).
void orc_bvh8_validate(const Node* nodes, uint32_t nn, const Tri* tris, uint32_t nt, const float* verts,
                       uint32_t ntris, uint32_t* info) {
    info[0] = info[1] = info[2] = 0;
    std::vector<uint32_t> seen(ntris, 0);
    struct Item { uint32_t node, depth; };
    std::vector<Item> st{{0, 1}};
    // returns bounds of a subtree (recursive through explicit stack: compute
    // geometry bounds per child by walking)
    std::function<bool(uint32_t, float*, float*, uint32_t)> walk;
    walk = [&](uint32_t ni, float* lo, float* hi, uint32_t depth) -> bool {
        if (ni >= nn) { info[2] = 1; return false; }
        info[0] = std::max(info[0], depth);
        const Node& N = nodes[ni];
        uint32_t k_int = 0, ntri_node = 0;
        for (int a = 0; a < 3; ++a) { lo[a] = INFINITY; hi[a] = -INFINITY; }
        for (int i = 0; i < 8; ++i) {
            uint32_t meta = N.meta[i];
            if (meta == 0) continue;
            float clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
            if ((N.imask >> i) & 1u) {
                if ((meta & 31u) != 24u + uint32_t(i) || (meta >> 5) != 1u) { info[2] = 5; return false; }
                if (!walk(N.child_base + k_int, clo, chi, depth + 1)) return false;
                k_int++;
            } else {
                uint32_t cnt = meta >> 5, off = meta & 31u;
                if (cnt != 1u && cnt != 3u && cnt != 7u) { info[2] = 5; return false; }
                uint32_t k = uint32_t(__builtin_popcount(cnt));
                ntri_node += k;
                for (uint32_t j = 0; j < k; ++j) {
                    uint32_t ti = N.tri_base + off + j;
                    if (ti >= nt) { info[2] = 1; return false; }
                    const Tri& T = tris[ti];
                    if (T.id >= ntris) { info[2] = 1; return false; }
                    seen[T.id]++;
                    const float* v = verts + 9ull * T.id;
                    const float* tv[3] = {T.v0, T.v1, T.v2};
                    for (int q = 0; q < 3; ++q)
                        for (int a = 0; a < 3; ++a) {
                            if (tv[q][a] != v[3 * q + a]) { info[2] = 4; return false; }
                            clo[a] = std::min(clo[a], tv[q][a]);
                            chi[a] = std::max(chi[a], tv[q][a]);
                        }
                }
            }
            for (int a = 0; a < 3; ++a) {
                double s = std::ldexp(1.0, N.ex[a]);
                double qlo = double(N.origin[a]) + N.qlo[a][i] * s, qhi = double(N.origin[a]) + N.qhi[a][i] * s;
                if (!(qlo <= clo[a] && qhi >= chi[a])) { info[2] = 2; return false; }
                lo[a] = std::min(lo[a], clo[a]);
                hi[a] = std::max(hi[a], chi[a]);
            }
        }
        info[1] = std::max(info[1], ntri_node);
        return true;
    };
    float lo[3], hi[3];
    if (!walk(0, lo, hi, 1)) return;
    for (uint32_t i = 0; i < ntris; ++i)
        if (seen[i] != 1u) { info[2] = 3; return; }
}

// Primary pass over a triangle BVH8 or a sphere list (ns > 0): visibility,
// FP32 t, and the reference g-buffer formats (depth R16F, normal RGBA16F,
// motion RG16F; any output may be NULL).
uint32_t orc_primary(const Node* nodes, uint32_t nn, const Tri* tris, uint32_t nt, const Mat* mats,
                     const float* spheres, uint32_t ns, const Consts* c, uint32_t w, uint32_t h, uint32_t y0,
                     uint32_t y1, uint32_t* vis, float* hit_t, uint16_t* depth, uint16_t* normal, uint16_t* motion,
                     int threads) {
    FrameInfo fi = frame_info(c, w, h);
    std::atomic<uint32_t> status{0};
    y1 = std::min(y1, h);
    if (y0 >= y1) return 0;
    parallel_rows(y1 - y0, threads, [&](uint32_t r, int) {
        const uint32_t y = y0 + r;
        uint32_t st = 0;
        for (uint32_t x = 0; x < w; ++x) {
            V3<float> o, d;
            primary_ray(fi, x, y, o, d);
            uint32_t prim = kMiss;
            float t = INFINITY;
            V3<float> n = d, pos = o;
            if (ns) {
                float tb = 0.0f;
                for (uint32_t i = 0; i < ns; ++i) {
                    const float* s = spheres + 8 * i;
                    float ts = ray_sphere(o, d, {s[0], s[1], s[2]}, s[3]);
                    if (ts >= 0.0f && (prim == kMiss || ts < tb)) { tb = ts; prim = i; }
                }
                if (prim != kMiss) {
                    const float* s = spheres + 8 * prim;
                    t = tb;
                    pos = o + d * tb;
                    n = normalize(pos - V3<float>{s[0], s[1], s[2]});
                }
            } else {
                Pre32 r = pre32(o, d);
                trace_bvh32(nodes, nn, tris, nt, r, 0.0f, INFINITY, false, prim, t, nullptr, &st);
                if (prim != kMiss) {
                    pos = o + d * t;
                    n = V3<float>{mats[prim].n[0], mats[prim].n[1], mats[prim].n[2]};
                    if (dot(n, d) > 0.0f) n = V3<float>{-n.x, -n.y, -n.z};
                }
            }
            size_t pi = size_t(y) * w + x;
            if (vis) vis[pi] = prim;
            if (hit_t) hit_t[pi] = t;
            float dep = 0.0f, mx = 0.0f, my = 0.0f;
            if (prim != kMiss) {
                float ph[4], pp[4];
                matvec(fi.pv, pos.x, pos.y, pos.z, 1.0f, ph);
                matvec(fi.ppv, pos.x, pos.y, pos.z, 1.0f, pp);
                float px = ph[0] / ph[3], py = ph[1] / ph[3];
                dep = ph[2] / ph[3];
                float qx = pp[0] / pp[3], qy = pp[1] / pp[3];
                mx = (px - qx) / fi.pitch_x;
                my = (py - qy) / fi.pitch_y;
            }
            if (depth) depth[pi] = f2h(dep);
            if (normal) {
                normal[4 * pi + 0] = f2h(n.x); normal[4 * pi + 1] = f2h(n.y);
                normal[4 * pi + 2] = f2h(n.z); normal[4 * pi + 3] = f2h(0.0f);
            }
            if (motion) { motion[2 * pi] = f2h(mx); motion[2 * pi + 1] = f2h(my); }
        }
        if (st) status.fetch_or(st);
    });
    return status.load();
}

// secondaryRays.comp:102-135 over a sphere list, from the g-buffer
// (visibility, R16F depth, RGBA16F normal); sky = the bound atmosphere
// (orc_sky_bind) or the constant radiance.
void orc_secondary_spheres(const float* spheres, uint32_t ns, const Consts* c, uint32_t w, uint32_t h,
                           const uint32_t* vis, const uint16_t* depth, const uint16_t* normal, const uint8_t* bn_rgba,
                           uint32_t bnw, uint32_t bnh, const Params* p, float* color, int threads) {
    FrameInfo fi = frame_info(c, w, h);
    const V3<float> sky{p->sky[0], p->sky[1], p->sky[2]};
    parallel_rows(h, threads, [&](uint32_t y, int) {
        for (uint32_t x = 0; x < w; ++x) {
            size_t pi = size_t(y) * w + x;
            float uvx = (float(x) + 0.5f) * fi.pitch_x;
            float uvy = 1.0f - (float(y) + 0.5f) * fi.pitch_y;
            uint32_t prim0 = vis[pi];
            V3<float> n0{h2f(normal[4 * pi]), h2f(normal[4 * pi + 1]), h2f(normal[4 * pi + 2])};
            float dep = h2f(depth[pi]);
            float vp[4], wp[4];
            matvec(c->inv_proj, uvx * 2.0f - 1.0f, uvy * 2.0f - 1.0f, dep, 1.0f, vp);
            vp[0] = vp[0] / vp[3]; vp[1] = vp[1] / vp[3]; vp[2] = vp[2] / vp[3];
            matvec(c->inv_view, vp[0], vp[1], vp[2], 1.0f, wp);
            V3<float> p0{wp[0], wp[1], wp[2]};
            uint32_t rng = initial_seed(p->rng_mode, c->frame, uint32_t(pi));
            size_t bi = size_t(y % bnh) * bnw + (x % bnw);
            float rotx = float(bn_rgba[4 * bi]) / 255.0f, roty = float(bn_rgba[4 * bi + 1]) / 255.0f;
            V3<float> acc{0, 0, 0};
            for (uint32_t s = 0; s < p->samples; ++s) {
                V3<float> col{1, 1, 1}, hp = p0, hn = n0, res{0, 0, 0};
                uint32_t hprim = prim0;
                for (uint32_t i = 0; i < p->max_bounces + 1u; ++i) {
                    if (i > 0) {
                        V3<float> ro = hp + hn * 0.000001f;
                        float u1 = rotated_random(rng, rotx);
                        float u2 = rotated_random(rng, roty);
                        V3<float> sp = sphere_point<float>(u1 * 2.0f - 1.0f, u2 * 2.0f - 1.0f);
                        V3<float> rd = normalize(hn + sp);
                        hprim = kMiss;
                        float ht = -1.0f;
                        for (uint32_t k = 0; k < ns; ++k) {
                            const float* sk = spheres + 8 * k;
                            float t = ray_sphere(ro, rd, {sk[0], sk[1], sk[2]}, sk[3]);
                            if (t >= 0.0f && (t < ht || ht < 0.0f)) { hprim = k; ht = t; }
                        }
                        if (hprim != kMiss) {
                            const float* sk = spheres + 8 * hprim;
                            hp = ro + rd * ht;
                            hn = normalize(hp - V3<float>{sk[0], sk[1], sk[2]});
                        } else hn = rd;
                    }
                    if (hprim != kMiss) {
                        const float* sk = spheres + 8 * hprim;
                        col = cmul(col, V3<float>{sk[4], sk[5], sk[6]});
                    } else {
                        res = cmul(col, escape32(sky, hn));
                        break;
                    }
                }
                acc = acc + res;
            }
            float nsf = float(p->samples);
            float* out = color + 3 * pi;
            float m[3] = {acc.x / nsf, acc.y / nsf, acc.z / nsf};
            for (int k = 0; k < 3; ++k) {
                if (p->accumulate && p->frame_index > 0u) m[k] = out[k] + (m[k] - out[k]) / float(p->frame_index + 1u);
                out[k] = m[k];
            }
        }
    });
}

// Batched bounce loop restated per ray for one scene: closest hits only,
// throughput x albedo, sky on escape, a PCG stream per ray seeded by its
// batch-wide index (index_base + i) and the frame, Russian roulette past
// rr_start.  radiance: 3 floats per ray.
uint32_t orc_pathtrace_rays(const Node* nodes, uint32_t nn, const Tri* tris, uint32_t nt, const Mat* mats,
                            const Ray* rays, uint32_t n, uint32_t index_base, const Params* p, uint32_t frame,
                            float* radiance, int threads) {
    std::atomic<uint32_t> status{0};
    const V3<float> sky{p->sky[0], p->sky[1], p->sky[2]};
    parallel_rows(n, threads, [&](uint32_t i, int) {
        uint32_t st = 0;
        const Ray& ry = rays[i];
        uint32_t h = (index_base + i) * 0x9E3779B1u + ((frame << 1u) | 1u);
        uint32_t rng = pcg(h) | 1u;
        V3<float> o{ry.o[0], ry.o[1], ry.o[2]}, d{ry.d[0], ry.d[1], ry.d[2]}, beta{1, 1, 1}, L{0, 0, 0};
        float tmax = ry.tmax;
        for (uint32_t v = 0;; ++v) {
            uint32_t prim;
            float t;
            Pre32 r = pre32(o, d);
            trace_bvh32(nodes, nn, tris, nt, r, 0.0f, tmax, false, prim, t, nullptr, &st);
            tmax = INFINITY;
            if (prim == kMiss) { L = cmul(beta, sky); break; }
            const Mat& m = mats[prim];
            V3<float> nrm{m.n[0], m.n[1], m.n[2]};
            if (dot(nrm, d) > 0.0f) nrm = V3<float>{-nrm.x, -nrm.y, -nrm.z};
            V3<float> rho{float(m.albedo & 0xFFu) / 255.0f, float((m.albedo >> 8) & 0xFFu) / 255.0f,
                          float((m.albedo >> 16) & 0xFFu) / 255.0f};
            beta = cmul(beta, rho);
            if (v >= p->max_bounces) break;
            float u1 = random_float(rng), u2 = random_float(rng);
            V3<float> sp = sphere_point<float>(u1 * 2.0f - 1.0f, u2 * 2.0f - 1.0f);
            V3<float> nd = nrm + sp;
            if (dot(nd, nd) == 0.0f) nd = nrm;
            nd = normalize(nd);
            if (p->rr_start != 0u && v + 1u > p->rr_start) {
                float q = std::fmin(std::fmax(std::fmax(std::fmax(beta.x, beta.y), beta.z), 0.05f), 1.0f);
                if (random_float(rng) >= q) break;
                beta = V3<float>{beta.x / q, beta.y / q, beta.z / q};
            }
            V3<float> hp = o + d * t;
            o = offset_ray(hp, nrm);
            d = nd;
        }
        radiance[3 * size_t(i)] = L.x;
        radiance[3 * size_t(i) + 1] = L.y;
        radiance[3 * size_t(i) + 2] = L.z;
        if (st) status.fetch_or(st);
    });
    return status.load();
}

// Triangle path tracer (the wavefront estimator, evaluated per pixel) from
// a primary visibility/t buffer; precision 32 or 64; rows [y0, y1) only
// (the rest of `color` is left untouched).  counts[0..2] += primary,
// extension, shadow rays.  Returns the status bits.
uint32_t orc_pathtrace(const Node* nodes, uint32_t nn, const Tri* tris, uint32_t nt, const Mat* mats, uint32_t nm,
                       const Consts* c, uint32_t w, uint32_t h, const uint32_t* vis, const float* hit_t,
                       const uint8_t* bn_rgba, uint32_t bnw, uint32_t bnh, const Params* p, int precision,
                       uint32_t y0, uint32_t y1, float* color, uint64_t* counts, int threads) {
    Scene sc{nodes, nn, tris, nt, mats, nm, nullptr, 0};
    FrameInfo fi = frame_info(c, w, h);
    std::vector<float> rot(size_t(bnw) * bnh * 2);
    for (size_t i = 0; i < size_t(bnw) * bnh; ++i) {
        rot[2 * i] = float(bn_rgba[4 * i]) / 255.0f;
        rot[2 * i + 1] = float(bn_rgba[4 * i + 1]) / 255.0f;
    }
    y1 = std::min(y1, h);
    if (y0 >= y1) return 0;
    std::atomic<uint64_t> cp{0}, ce{0}, cs{0};
    std::atomic<uint32_t> status{0};
    parallel_rows(y1 - y0, threads, [&](uint32_t r, int) {
        uint32_t y = y0 + r;
        RayCounts rc;
        uint32_t st = 0;
        for (uint32_t x = 0; x < w; ++x) {
            size_t pi = size_t(y) * w + x;
            float m[3];
            if (precision == 64) {
                // FP64 primary hit from the FP32 visibility; t re-solved in double
                uint32_t prim = vis[pi];
                double t0 = 0.0;
                if (prim != kMiss) {
                    V3<double> o, d;
                    primary_ray_d(fi, x, y, o, d);
                    uint32_t pp;
                    trace_bvh64(nodes, nn, tris, nt, o, d, 0.0, INFINITY, false, pp, t0);
                    prim = pp;
                }
                V3<double> L = shade_pixel<double>(sc, fi, *p, rot.data(), bnw, bnh, x, y, prim, t0, rc, &st);
                m[0] = float(L.x / p->samples); m[1] = float(L.y / p->samples); m[2] = float(L.z / p->samples);
            } else {
                V3<float> L = shade_pixel<float>(sc, fi, *p, rot.data(), bnw, bnh, x, y, vis[pi], hit_t[pi], rc, &st);
                float nsf = float(p->samples);
                m[0] = L.x / nsf; m[1] = L.y / nsf; m[2] = L.z / nsf;
            }
            float* out = color + 3 * pi;
            for (int k = 0; k < 3; ++k) {
                if (p->accumulate && p->frame_index > 0u) m[k] = out[k] + (m[k] - out[k]) / float(p->frame_index + 1u);
                out[k] = m[k];
            }
            rc.primary++;
        }
        cp += rc.primary; ce += rc.ext; cs += rc.shadow;
        if (st) status.fetch_or(st);
    });
    if (counts) { counts[0] += cp.load(); counts[1] += ce.load(); counts[2] += cs.load(); }
    return status.load();
}

} // extern "C"

// ---- temporal reprojection (new; mirrors the CUDA kernel's definition) ----
// History read bilinearly at this pixel's previous-frame position (its
// motion vector), taps kept when the previous frame saw a surface with an
// agreeing normal and linear depth; n = min(n_prev + 1, max_history); the
// result is history + (sample - history) / n; n = 1 when nothing survives.
extern "C" void orc_reproject(const Consts* c, uint32_t w, uint32_t h, const uint32_t* vis, const float* hit_t,
                              const uint16_t* normal, const uint16_t* motion, const uint32_t* pvis,
                              const uint16_t* pdepth, const uint16_t* pnormal, const float* sample,
                              const float* hist, const float* hist_len, float max_history, float normal_cos,
                              float depth_rel, float* out, float* out_len) {
    const FrameInfo fi = frame_info(c, w, h);
    const float near_plane = c->proj[3 * 4 + 2];
    for (uint32_t y = 0; y < h; ++y)
        for (uint32_t x = 0; x < w; ++x) {
            const size_t i = size_t(y) * w + x;
            V3<float> res{sample[3 * i], sample[3 * i + 1], sample[3 * i + 2]};
            const V3<float> s = res;
            float len = 1.0f;
            if (vis[i] != kMiss) {
                const float px = (float(x) + 0.5f) - h2f(motion[2 * i]) * 0.5f;
                const float py = (float(y) + 0.5f) + h2f(motion[2 * i + 1]) * 0.5f;
                V3<float> o, d;
                primary_ray(fi, x, y, o, d);
                const V3<float> p = o + d * hit_t[i];
                float q[4];
                matvec(fi.ppv, p.x, p.y, p.z, 1.0f, q);
                const float exp_lin = q[3];
                const V3<float> cn{h2f(normal[4 * i]), h2f(normal[4 * i + 1]), h2f(normal[4 * i + 2])};
                const float fx = px - 0.5f, fy = py - 0.5f;
                const float x0 = std::floor(fx), y0 = std::floor(fy);
                if (exp_lin > 0.0f && x0 >= -1.0f && x0 <= float(w) - 1.0f && y0 >= -1.0f && y0 <= float(h) - 1.0f) {
                    const float wx = fx - x0, wy = fy - y0, gx = 1.0f - wx, gy = 1.0f - wy;
                    const float ws[4] = {gx * gy, wx * gy, gx * wy, wx * wy};
                    const float tol = depth_rel * exp_lin;
                    float sw = 0.0f, hl = 0.0f;
                    V3<float> hh{0.0f, 0.0f, 0.0f};
                    for (int t = 0; t < 4; ++t) {
                        const int tx = int(x0) + (t & 1), ty = int(y0) + (t >> 1);
                        if (tx < 0 || ty < 0 || tx >= int(w) || ty >= int(h) || !(ws[t] > 0.0f)) continue;
                        const size_t j = size_t(ty) * w + tx;
                        if (pvis[j] == kMiss) continue;
                        const V3<float> pn{h2f(pnormal[4 * j]), h2f(pnormal[4 * j + 1]), h2f(pnormal[4 * j + 2])};
                        if (!(dot(pn, cn) >= normal_cos)) continue;
                        const float tl = near_plane / h2f(pdepth[j]);
                        if (!(std::fabs(tl - exp_lin) <= tol)) continue;
                        sw = sw + ws[t];
                        hh = hh + V3<float>{hist[3 * j], hist[3 * j + 1], hist[3 * j + 2]} * ws[t];
                        hl = hl + hist_len[j] * ws[t];
                    }
                    if (sw > 0.0f) {
                        hh = V3<float>{hh.x / sw, hh.y / sw, hh.z / sw};
                        len = std::fmin(hl / sw + 1.0f, max_history);
                        const float a = 1.0f / len;
                        res = hh + (s - hh) * a;
                    }
                }
            }
            out[3 * i] = res.x;
            out[3 * i + 1] = res.y;
            out[3 * i + 2] = res.z;
            out_len[i] = len;
        }
}
