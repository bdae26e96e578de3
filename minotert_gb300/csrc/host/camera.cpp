// Camera math of the renderer's host side: view / projection / inverse and
// the per-dispatch constant fill.  Follows the reference's semantics:
//   Camera::direction/view/projection   src/gfx/camera.ixx:19-44
//   look / perspective                  src/stx/math.ixx:822-861
//   inverse (4x4 cofactor expansion)    src/stx/math.ixx:739-820
//   constants fill                      src/gfx/modules/pathtracer.ixx:86-105, 171-184
// Arithmetic is plain IEEE float with no contraction (built with
// -ffp-contract=off), with the reference's operation order, so the values
// are reproducible on every host.
#include "mrt_host.h"

#include <cmath>
#include <cstring>

namespace {

struct V3 { float x, y, z; };

inline float dot3(V3 a, V3 b) {
    // minote.math dot: result = 0; result += a[i]*b[i] in index order
    float r = 0.0f;
    r += a.x * b.x;
    r += a.y * b.y;
    r += a.z * b.z;
    return r;
}

inline V3 cross3(V3 l, V3 r) {
    return V3{l.y * r.z - r.y * l.z, l.z * r.x - r.z * l.x, l.x * r.y - r.x * l.y};
}

inline V3 normalize3(V3 v) {
    float len = std::sqrt(dot3(v, v));
    return V3{v.x / len, v.y / len, v.z / len};
}

// column-major element access: m[col*4 + row]
// sin / cos / tan of a binary32 angle, evaluated in binary64 and rounded
// once, so the matrices have the same bits on every host
inline float sin_(float x) { return float(std::sin(double(x))); }
inline float cos_(float x) { return float(std::cos(double(x))); }
inline float tan_(float x) { return float(std::tan(double(x))); }

inline float& el(float* m, int col, int row) { return m[col * 4 + row]; }
inline float el(const float* m, int col, int row) { return m[col * 4 + row]; }

void look(V3 pos, V3 dir, V3 up, float* out) {
    for (int i = 0; i < 16; ++i) out[i] = (i % 5 == 0) ? 1.0f : 0.0f;
    V3 s = normalize3(cross3(up, dir));
    V3 u = cross3(dir, s);
    el(out, 0, 0) = -s.x; el(out, 1, 0) = -s.y; el(out, 2, 0) = -s.z;
    el(out, 0, 1) = u.x;  el(out, 1, 1) = u.y;  el(out, 2, 1) = u.z;
    el(out, 0, 2) = dir.x; el(out, 1, 2) = dir.y; el(out, 2, 2) = dir.z;
    el(out, 3, 0) = dot3(s, pos);
    el(out, 3, 1) = -dot3(u, pos);
    el(out, 3, 2) = -dot3(dir, pos);
}

void perspective(float vfov, float aspect, float znear, float* out) {
    float h = 1.0f / tan_(0.5f * vfov);
    float w = h * aspect;
    for (int i = 0; i < 16; ++i) out[i] = 0.0f;
    el(out, 0, 0) = w;
    el(out, 1, 1) = h;
    el(out, 2, 3) = 1.0f;
    el(out, 3, 2) = znear;
}

} // namespace

extern "C" {

void mrt_camera_view(const mrt_camera* cam, float out[16]) {
    float cp = cos_(cam->pitch), sp = sin_(cam->pitch);
    float cy = cos_(cam->yaw), sy = sin_(cam->yaw);
    V3 dir{cp * cy, cp * sy, sp};
    look(V3{cam->position[0], cam->position[1], cam->position[2]}, dir, V3{0.0f, 0.0f, 1.0f}, out);
}

void mrt_camera_projection(const mrt_camera* cam, float out[16]) {
    perspective(cam->vertical_fov, float(cam->viewport[1]) / float(cam->viewport[0]),
                cam->near_plane, out);
}

void mrt_mat4_inverse(const float* m, float* out) {
    // Cofactor pairs of the 2x2 minors in columns 2-3 / 1-3 / 1-2 (the
    // expansion of math.ixx:761-818, same operation order).
    auto minor = [&](int c0, int c1, int ra, int rb) {
        return el(m, c0, ra) * el(m, c1, rb) - el(m, c1, ra) * el(m, c0, rb);
    };
    // coefficient blocks indexed [block][k]: block b uses rows (ra, rb)
    // against columns pairs of the reference's coef00..coef23
    float c00 = minor(2, 3, 2, 3), c02 = minor(1, 3, 2, 3), c03 = minor(1, 2, 2, 3);
    float c04 = minor(2, 3, 1, 3), c06 = minor(1, 3, 1, 3), c07 = minor(1, 2, 1, 3);
    float c08 = minor(2, 3, 1, 2), c10 = minor(1, 3, 1, 2), c11 = minor(1, 2, 1, 2);
    float c12 = minor(2, 3, 0, 3), c14 = minor(1, 3, 0, 3), c15 = minor(1, 2, 0, 3);
    float c16 = minor(2, 3, 0, 2), c18 = minor(1, 3, 0, 2), c19 = minor(1, 2, 0, 2);
    float c20 = minor(2, 3, 0, 1), c22 = minor(1, 3, 0, 1), c23 = minor(1, 2, 0, 1);

    const float fac[6][4] = {
        {c00, c00, c02, c03}, {c04, c04, c06, c07}, {c08, c08, c10, c11},
        {c12, c12, c14, c15}, {c16, c16, c18, c19}, {c20, c20, c22, c23}};
    float v[4][4]; // v[r][k] = {m[1][r], m[0][r], m[0][r], m[0][r]}
    for (int r = 0; r < 4; ++r) {
        v[r][0] = el(m, 1, r);
        v[r][1] = v[r][2] = v[r][3] = el(m, 0, r);
    }
    // inv_c = va*fa - vb*fb + vc*fc (component-wise), then signs
    const int terms[4][3][2] = {
        {{1, 0}, {2, 1}, {3, 2}}, // inv0 = v1*fac0 - v2*fac1 + v3*fac2
        {{0, 0}, {2, 3}, {3, 4}}, // inv1 = v0*fac0 - v2*fac3 + v3*fac4
        {{0, 1}, {1, 3}, {3, 5}}, // inv2 = v0*fac1 - v1*fac3 + v3*fac5
        {{0, 2}, {1, 4}, {2, 5}}, // inv3 = v0*fac2 - v1*fac4 + v2*fac5
    };
    float inv[4][4];
    for (int c = 0; c < 4; ++c) {
        for (int k = 0; k < 4; ++k) {
            float a = v[terms[c][0][0]][k] * fac[terms[c][0][1]][k];
            float b = v[terms[c][1][0]][k] * fac[terms[c][1][1]][k];
            float d = v[terms[c][2][0]][k] * fac[terms[c][2][1]][k];
            float val = a - b + d;
            // signA = {+,-,+,-} for columns 0,2; signB = {-,+,-,+} for 1,3
            bool neg = ((c & 1) == 0) ? (k & 1) : !(k & 1);
            inv[c][k] = neg ? -val : val;
        }
    }
    // determinant from column 0 of m against row 0 of inv
    float d0 = el(m, 0, 0) * inv[0][0];
    float d1 = el(m, 0, 1) * inv[1][0];
    float d2 = el(m, 0, 2) * inv[2][0];
    float d3 = el(m, 0, 3) * inv[3][0];
    float det = (d0 + d1) + (d2 + d3);
    float one_over = 1.0f / det;
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) el(out, c, r) = inv[c][r] * one_over;
}

void mrt_camera_consts_make(const mrt_camera* cam, const mrt_camera* prev_cam,
                            uint32_t frame_counter, mrt_camera_consts* out) {
    std::memset(out, 0, sizeof(*out));
    mrt_camera_view(cam, out->view);
    mrt_camera_projection(cam, out->projection);
    mrt_mat4_inverse(out->view, out->inv_view);
    mrt_mat4_inverse(out->projection, out->inv_projection);
    mrt_camera_view(prev_cam ? prev_cam : cam, out->prev_view);
    out->camera_pos[0] = cam->position[0];
    out->camera_pos[1] = cam->position[1];
    out->camera_pos[2] = cam->position[2];
    out->frame_counter = frame_counter;
}

uint32_t mrt_scene_reference(mrt_sphere* out) {
    // scene.glsl:4-11, km units
    static const float s[5][7] = {
        {0.0000f, 0.0017f, 0.10000f, 0.00050f, 0.2f, 0.7f, 0.0f},
        {-0.0008f, 0.0012f, 0.09983f, 0.00033f, 0.0f, 0.2f, 0.7f},
        {0.0008f, 0.0012f, 0.09983f, 0.00033f, 0.7f, 0.0f, 0.2f},
        {0.0000f, 0.0008f, 0.09975f, 0.00025f, 1.0f, 1.0f, 1.0f},
        {0.0000f, 0.0010f, -0.00050f, 0.10000f, 0.5f, 0.5f, 0.5f},
    };
    if (out) {
        for (int i = 0; i < 5; ++i) {
            out[i].center[0] = s[i][0]; out[i].center[1] = s[i][1]; out[i].center[2] = s[i][2];
            out[i].radius = s[i][3];
            out[i].albedo[0] = s[i][4]; out[i].albedo[1] = s[i][5]; out[i].albedo[2] = s[i][6];
            out[i].pad = 0.0f;
        }
    }
    return 5;
}

void mrt_camera_reference(uint32_t width, uint32_t height, mrt_camera* out) {
    // app.ixx:20-32: 60 degree vertical fov, near 1 mm, at (0,-1 m,100 m),
    // yaw 90 degrees (looking along +Y), level pitch.
    out->viewport[0] = width;
    out->viewport[1] = height;
    out->vertical_fov = float(60.0 * 3.14159265358979323846 / 180.0);
    out->near_plane = 0.001f;
    out->position[0] = 0.0f; out->position[1] = -0.001f; out->position[2] = 0.1f;
    out->yaw = float(90.0 * 3.14159265358979323846 / 180.0);
    out->pitch = 0.0f;
}

} // extern "C"
