// CPU restatement of the headless half-angle slice renderer -- TEST INFRASTRUCTURE ONLY (the
// checker of smk_render; nothing in the library calls it).
//
// It restates the reference's two-pass volume drawing (project/main.cpp:369-419, 474-476,
// 660-661, 676-687; texVolume.frag:27-52; light.frag:16-23; proxy planes of boundingBox.cpp:
// 135-181, 228-345) as plain loops, in the operation order smk_render uses:
//   - plane i of P sits at start + (end - start) * ((i + 0.5) / P) with normal n = the unit half
//     vector (-cam_dir + light_dir when camera and light face each other); start/end are the
//     extreme projections of the box corners (+-dimensions/2 about the world origin) on n;
//   - drawing order: for every plane, the eye pass (reads the light buffer after the previous
//     plane) then the light pass;
//   - a pixel/texel sees plane i where its ray meets the plane, if that point is in the box and
//     its ray parameter is within [near, far];
//   - density: trilinear, clamp to edge, coordinate ((p - box) / (n / 2) + 1) / 2 (integer n/2);
//     light colour: bilinear, repeat, at the point's light-view NDC mapped to [0, 1];
//   - blends: eye front-to-back (ONE_MINUS_DST_ALPHA, ONE) on (c * a, a), or back-to-front
//     (SRC_ALPHA, ONE_MINUS_SRC_ALPHA) / (ONE, ONE_MINUS_SRC_ALPHA) on (c, a); light
//     (SRC_ALPHA, ONE_MINUS_SRC_ALPHA) / (ONE, ONE_MINUS_SRC_ALPHA) on (0, 0, 0, a);
//   - every stored framebuffer value is rounded to half precision (RGBA16F), round to nearest
//     even, converted here from the IEEE 754 binary16 definition.
// GL rasterisation and the texture unit's fixed-point filter weights are not reproduced: parity
// with an OpenGL run is unpinned (no graphics stack on the build machines); this restatement is
// the definition smk_render is checked against, bit for bit.
// Build: g++ -O2 -ffp-contract=off (oracle/build_oracle.py).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

extern "C" {
typedef struct {
    int width, height, light_res, planes;
    float camera_pos[3], camera_dir[3], up[3];
    float fovy_deg, znear, zfar;
    float light_pos[3];
    float light_fovy_deg, light_znear, light_zfar;
    float light_color[3];
    float box_pos[3];
    float cell_size;
    float bg_color[3];
} orc_render_params;
}

namespace {

struct V3 {
    float x, y, z;
};
inline V3 mk(float x, float y, float z) { return V3{x, y, z}; }
inline V3 add(V3 a, V3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 sub(V3 a, V3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 scl(V3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
inline float dot3(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross3(V3 a, V3 b) { return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
inline V3 norm3(V3 a) { return scl(a, 1.0f / std::sqrt(dot3(a, a))); }

// IEEE 754 binary32 -> binary16, round to nearest, ties to even (overflow to infinity).
uint16_t to_half(float f) {
    uint32_t x;
    std::memcpy(&x, &f, 4);
    const uint32_t sign = (x >> 16) & 0x8000u;
    const uint32_t exp = (x >> 23) & 0xffu;
    uint32_t mant = x & 0x7fffffu;
    if (exp == 0xffu) return (uint16_t)(sign | 0x7c00u | (mant ? 0x200u : 0u));
    const int e = (int)exp - 127 + 15;
    if (e >= 31) return (uint16_t)(sign | 0x7c00u);
    if (e <= 0) {
        if (e < -10) return (uint16_t)sign;
        mant |= 0x800000u;
        const int shift = 14 - e;
        uint32_t h = mant >> shift;
        const uint32_t rem = mant & ((1u << shift) - 1u), halfway = 1u << (shift - 1);
        if (rem > halfway || (rem == halfway && (h & 1u))) ++h;
        return (uint16_t)(sign | h);
    }
    uint32_t h = sign | ((uint32_t)e << 10) | (mant >> 13);
    const uint32_t rem = mant & 0x1fffu;
    if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) ++h;  // a carry into the exponent is correct
    return (uint16_t)h;
}

float from_half(uint16_t h) {
    const uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
    const int exp = (h >> 10) & 0x1f;
    const uint32_t mant = h & 0x3ffu;
    float v;
    if (exp == 0) v = std::ldexp((float)mant, -24);
    else if (exp == 31) v = mant ? NAN : INFINITY;
    else v = std::ldexp((float)(mant | 0x400u), exp - 25);
    uint32_t b;
    std::memcpy(&b, &v, 4);
    b |= sign;
    std::memcpy(&v, &b, 4);
    return v;
}

inline float h16(float x) { return from_half(to_half(x)); }

struct View {
    V3 eye, s, u, f;
    float sx, sy, znear, zfar;
    int w, h;
};

View make_view(V3 eye, V3 dir, V3 up, float fovy_deg, float aspect, float zn, float zf, int w, int h) {
    View v;
    v.eye = eye;
    v.f = norm3(dir);
    v.s = norm3(cross3(v.f, up));
    v.u = cross3(v.s, v.f);
    const float th = (float)std::tan(0.5 * (double)fovy_deg * 3.14159265358979323846 / 180.0);
    v.sx = aspect * th;
    v.sy = th;
    v.znear = zn;
    v.zfar = zf;
    v.w = w;
    v.h = h;
    return v;
}

struct Scene {
    View cam, light;
    V3 start, end, n, box_min, box_max, box_pos, tex_half;
    int planes, back_to_front, nx, ny, nz;
    float clear[4], bg[3];
    const float* rho;
};

V3 ray_dir(const View& V, int px, int py) {
    const float nx = (2.0f * ((float)px + 0.5f)) / (float)V.w - 1.0f;
    const float ny = (2.0f * ((float)py + 0.5f)) / (float)V.h - 1.0f;
    return add(add(V.f, scl(V.s, nx * V.sx)), scl(V.u, ny * V.sy));
}

bool hit(const Scene& S, const View& V, V3 d, float denom, int i, V3* p) {
    if (denom == 0.0f) return false;
    const float ti = ((float)i + 0.5f) / (float)S.planes;
    const V3 pp = add(S.start, scl(sub(S.end, S.start), ti));
    const float t = dot3(sub(pp, V.eye), S.n) / denom;
    if (!(t >= V.znear && t <= V.zfar)) return false;
    *p = add(V.eye, scl(d, t));
    return p->x >= S.box_min.x && p->x <= S.box_max.x && p->y >= S.box_min.y && p->y <= S.box_max.y &&
           p->z >= S.box_min.z && p->z <= S.box_max.z;
}

inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

float cell(const Scene& S, int x, int y, int z) { return S.rho[(size_t)x + (size_t)S.nx * (y + (size_t)S.ny * z)]; }

float density(const Scene& S, V3 p) {
    const float tx = ((p.x - S.box_pos.x) / S.tex_half.x + 1.0f) / 2.0f;
    const float ty = ((p.y - S.box_pos.y) / S.tex_half.y + 1.0f) / 2.0f;
    const float tz = ((p.z - S.box_pos.z) / S.tex_half.z + 1.0f) / 2.0f;
    const float ux = tx * (float)S.nx - 0.5f, uy = ty * (float)S.ny - 0.5f, uz = tz * (float)S.nz - 0.5f;
    const float fx = std::floor(ux), fy = std::floor(uy), fz = std::floor(uz);
    const float ax = ux - fx, ay = uy - fy, az = uz - fz;
    const int x0 = clampi((int)fx, 0, S.nx - 1), x1 = clampi((int)fx + 1, 0, S.nx - 1);
    const int y0 = clampi((int)fy, 0, S.ny - 1), y1 = clampi((int)fy + 1, 0, S.ny - 1);
    const int z0 = clampi((int)fz, 0, S.nz - 1), z1 = clampi((int)fz + 1, 0, S.nz - 1);
    const float c00 = cell(S, x0, y0, z0) * (1.0f - ax) + cell(S, x1, y0, z0) * ax;
    const float c10 = cell(S, x0, y1, z0) * (1.0f - ax) + cell(S, x1, y1, z0) * ax;
    const float c01 = cell(S, x0, y0, z1) * (1.0f - ax) + cell(S, x1, y0, z1) * ax;
    const float c11 = cell(S, x0, y1, z1) * (1.0f - ax) + cell(S, x1, y1, z1) * ax;
    const float c0 = c00 * (1.0f - ay) + c10 * ay;
    const float c1 = c01 * (1.0f - ay) + c11 * ay;
    return c0 * (1.0f - az) + c1 * az;
}

inline int wrapi(int v, int n) {
    const int r = v % n;
    return r < 0 ? r + n : r;
}

void light_lookup(const std::vector<uint16_t>& L, int R, float u, float v, float out[4]) {
    const float sx = std::fmin(std::fmax(u * (float)R - 0.5f, -1.0e6f), 1.0e6f);
    const float sy = std::fmin(std::fmax(v * (float)R - 0.5f, -1.0e6f), 1.0e6f);
    const float fx = std::floor(sx), fy = std::floor(sy);
    const float ax = sx - fx, ay = sy - fy;
    const int x0 = wrapi((int)fx, R), x1 = wrapi((int)fx + 1, R);
    const int y0 = wrapi((int)fy, R), y1 = wrapi((int)fy + 1, R);
    for (int c = 0; c < 4; ++c) {
        const float t00 = from_half(L[4 * (x0 + R * y0) + c]), t10 = from_half(L[4 * (x1 + R * y0) + c]);
        const float t01 = from_half(L[4 * (x0 + R * y1) + c]), t11 = from_half(L[4 * (x1 + R * y1) + c]);
        out[c] = (t00 * (1.0f - ax) + t10 * ax) * (1.0f - ay) + (t01 * (1.0f - ax) + t11 * ax) * ay;
    }
}

}  // namespace

extern "C" {

// rho: nx*ny*nz densities (x fastest); eye_rgba: width*height*4; comp_rgb: width*height*3 or
// NULL; rows bottom-up.  Returns 0.
int orc_render(const float* rho, int nx, int ny, int nz, const orc_render_params* rp, float* eye_rgba,
               float* comp_rgb) {
    Scene S;
    S.rho = rho;
    S.nx = nx;
    S.ny = ny;
    S.nz = nz;
    const V3 cam = mk(rp->camera_pos[0], rp->camera_pos[1], rp->camera_pos[2]);
    const V3 up = mk(rp->up[0], rp->up[1], rp->up[2]);
    const V3 lp = mk(rp->light_pos[0], rp->light_pos[1], rp->light_pos[2]);
    const V3 box = mk(rp->box_pos[0], rp->box_pos[1], rp->box_pos[2]);
    S.cam = make_view(cam, mk(rp->camera_dir[0], rp->camera_dir[1], rp->camera_dir[2]), up, rp->fovy_deg,
                      (float)rp->width / (float)rp->height, rp->znear, rp->zfar, rp->width, rp->height);
    S.light = make_view(lp, sub(box, lp), up, rp->light_fovy_deg, 1.0f, rp->light_znear, rp->light_zfar,
                        rp->light_res, rp->light_res);
    const V3 cam_view = sub(box, cam), light_view = sub(box, lp);
    const V3 cn = norm3(cam_view), ln = norm3(light_view);
    V3 half = add(cn, ln);
    if (dot3(cn, ln) < 0.0f) half = add(mk(-cn.x, -cn.y, -cn.z), ln);
    S.back_to_front = dot3(cam_view, light_view) < 0.0f ? 1 : 0;
    const V3 dims = mk(rp->cell_size * nx, rp->cell_size * ny, rp->cell_size * nz);
    const V3 hd = scl(dims, 0.5f);
    S.n = norm3(half);
    float mn = 0.0f, mx = 0.0f;
    for (int c = 0; c < 8; ++c) {
        const V3 corner = mk((c & 1) ? hd.x : -hd.x, (c & 2) ? hd.y : -hd.y, (c & 4) ? hd.z : -hd.z);
        const float d = dot3(corner, S.n);
        if (c == 0 || d < mn) mn = d;
        if (c == 0 || d > mx) mx = d;
    }
    S.start = scl(S.n, mn);
    S.end = scl(S.n, mx);
    S.planes = rp->planes;
    S.box_pos = box;
    S.box_min = sub(box, hd);
    S.box_max = add(box, hd);
    S.tex_half = mk((float)(nx / 2), (float)(ny / 2), (float)(nz / 2));
    for (int k = 0; k < 3; ++k) {
        S.clear[k] = h16(rp->light_color[k]);
        S.bg[k] = rp->bg_color[k];
    }
    S.clear[3] = 1.0f;

    // light buffer after every plane
    const int R = rp->light_res;
    std::vector<std::vector<uint16_t>> slices(S.planes, std::vector<uint16_t>((size_t)R * R * 4));
    for (int ly = 0; ly < R; ++ly)
        for (int lx = 0; lx < R; ++lx) {
            const V3 d = ray_dir(S.light, lx, ly);
            const float denom = dot3(d, S.n);
            float c[4] = {S.clear[0], S.clear[1], S.clear[2], S.clear[3]};
            for (int i = 0; i < S.planes; ++i) {
                V3 p;
                if (hit(S, S.light, d, denom, i, &p)) {
                    const float a = density(S, p);
                    const float om = 1.0f - a;
                    c[0] = h16(c[0] * om);
                    c[1] = h16(c[1] * om);
                    c[2] = h16(c[2] * om);
                    c[3] = h16(a + c[3] * om);
                }
                for (int k = 0; k < 4; ++k) slices[i][4 * ((size_t)lx + (size_t)R * ly) + k] = to_half(c[k]);
            }
        }
    // eye buffer
    const int W = rp->width, H = rp->height;
    for (int py = 0; py < H; ++py)
        for (int px = 0; px < W; ++px) {
            const V3 d = ray_dir(S.cam, px, py);
            const float denom = dot3(d, S.n);
            float e[4] = {0.0f, 0.0f, 0.0f, 0.0f};
            for (int i = 0; i < S.planes; ++i) {
                V3 p;
                if (!hit(S, S.cam, d, denom, i, &p)) continue;
                const float a = density(S, p);
                float lc[4] = {S.clear[0], S.clear[1], S.clear[2], S.clear[3]};
                if (i > 0) {
                    const V3 q = sub(p, S.light.eye);
                    const float depth = dot3(q, S.light.f);
                    const float u = (dot3(q, S.light.s) / (S.light.sx * depth)) * 0.5f + 0.5f;
                    const float v = (dot3(q, S.light.u) / (S.light.sy * depth)) * 0.5f + 0.5f;
                    light_lookup(slices[i - 1], R, u, v, lc);
                }
                if (S.back_to_front) {
                    const float om = 1.0f - a;
                    e[0] = h16(lc[0] * a + e[0] * om);
                    e[1] = h16(lc[1] * a + e[1] * om);
                    e[2] = h16(lc[2] * a + e[2] * om);
                    e[3] = h16(a + e[3] * om);
                } else {
                    const float om = 1.0f - e[3];
                    e[0] = h16((lc[0] * a) * om + e[0]);
                    e[1] = h16((lc[1] * a) * om + e[1]);
                    e[2] = h16((lc[2] * a) * om + e[2]);
                    e[3] = h16(a * om + e[3]);
                }
            }
            const size_t id = (size_t)px + (size_t)W * py;
            for (int k = 0; k < 4; ++k) eye_rgba[4 * id + k] = e[k];
            if (comp_rgb) {
                const float om = 1.0f - e[3];
                for (int k = 0; k < 3; ++k) comp_rgb[3 * id + k] = e[k] * e[3] + S.bg[k] * om;
            }
        }
    return 0;
}

// Proxy-plane polygons (boundingBox.cpp:87-92, 133-181, 231-360), the checker of
// smk_proxy_planes, in the reference's own order of operations: d1 = normalize(-view_dir) (the
// ray direction); getMinMaxPoints and sortPoints normalise it once more (d2 = normalize(d1));
// the extreme projections of the box corners vec3(+-1,+-1,+-1) * dims / 2 (about the world
// origin) on d2 give start = origin + d1 * min and end = origin + d1 * max; plane i (step
// i + 0.5) lies at start + (end - start) * (step / planes), normal d1; the box's 12 edges (X
// edges for y, z in {-1, 1}, then Y edges for x, z, then Z edges for y, x) are intersected with
// it (t = dot(o - ro, d1) / dot(rd, d1), kept when 0 <= t <= edge length; edges parallel to the
// plane are skipped), exact repeats dropped; the centroid is the sum divided by the count; the
// points are sorted by pseudo-angle about it (ax = normalize(p0 - c), ay = cross(d2, ax), key
// 1 + r below the ax axis, 3 - r above, evaluated in double as the reference's literals are),
// descending, by a stable insertion sort (std::sort's order on the at most 6 points); fan
// triangulation.  Output layout as smk_proxy_planes.
static float proxy_key(float x, float y) {
    const float r = x / (std::fabs(x) + std::fabs(y));
    if (y < 0.0f) return (float)(1.0 + (double)r);
    return (float)(3.0 - (double)r);
}

int orc_proxy_planes(const float* view_origin, const float* view_dir, const float* box_pos, const float* dims,
                     int planes, float* verts, int* counts, int* tris) {
    const V3 d1 = norm3(mk(-view_dir[0], -view_dir[1], -view_dir[2]));
    const V3 d2 = norm3(d1);
    const V3 box = mk(box_pos[0], box_pos[1], box_pos[2]);
    const V3 dm = mk(dims[0], dims[1], dims[2]);
    const V3 half = mk(dm.x / 2.0f, dm.y / 2.0f, dm.z / 2.0f);
    const V3 vo = mk(view_origin[0], view_origin[1], view_origin[2]);
    static const float corner_sign[8][3] = {{-1, -1, 1}, {1, -1, 1}, {-1, 1, 1}, {1, 1, 1},
                                            {-1, -1, -1}, {1, -1, -1}, {-1, 1, -1}, {1, 1, -1}};
    float mn = 0.0f, mx = 0.0f;
    for (int c = 0; c < 8; ++c) {
        const V3 corner = mk(corner_sign[c][0] * dm.x / 2.0f, corner_sign[c][1] * dm.y / 2.0f,
                             corner_sign[c][2] * dm.z / 2.0f);
        const float dd = dot3(sub(corner, vo), d2);
        if (c == 0) mn = mx = dd;
        if (dd < mn) mn = dd;
        if (dd > mx) mx = dd;
    }
    const V3 start = add(vo, scl(d1, mn)), end = add(vo, scl(d1, mx));
    const int MAXP = 7;
    for (int i = 0; i < planes; ++i) {
        const float t = ((float)i + 0.5f) / (float)planes;
        const V3 o = add(start, scl(sub(end, start), t));
        std::vector<V3> pts;
        V3 c = mk(0.0f, 0.0f, 0.0f);
        for (int axis = 0; axis < 3; ++axis)
            for (int a = -1; a < 2; a += 2)
                for (int b = -1; b < 2; b += 2) {
                    V3 ro, rd;
                    float len;
                    if (axis == 0) {
                        ro = sub(box, mk(half.x, half.y * (float)a, half.z * (float)b));
                        rd = mk(1.0f, 0.0f, 0.0f);
                        len = dm.x;
                    } else if (axis == 1) {
                        ro = sub(box, mk(half.x * (float)a, half.y, half.z * (float)b));
                        rd = mk(0.0f, 1.0f, 0.0f);
                        len = dm.y;
                    } else {
                        ro = sub(box, mk(half.x * (float)b, half.y * (float)a, half.z));
                        rd = mk(0.0f, 0.0f, 1.0f);
                        len = dm.z;
                    }
                    const float den = dot3(rd, d1);
                    if (den == 0.0f) continue;
                    const float tt = dot3(sub(o, ro), d1) / den;
                    if (tt > len || tt < 0.0f) continue;
                    const V3 p = add(ro, scl(rd, tt));
                    bool dup = false;
                    for (const V3& q : pts) dup = dup || (p.x == q.x && p.y == q.y && p.z == q.z);
                    if (!dup && (int)pts.size() < MAXP - 1) {
                        pts.push_back(p);
                        c = add(c, p);
                    }
                }
        const int k = (int)pts.size();
        if (k > 0) c = mk(c.x / (float)k, c.y / (float)k, c.z / (float)k);
        if (k > 0) {
            const V3 ax = norm3(sub(pts[0], c));
            const V3 ay = cross3(d2, ax);
            std::vector<float> key(k);
            for (int q = 0; q < k; ++q) {
                const V3 v = sub(pts[q], c);
                key[q] = proxy_key(dot3(ax, v), dot3(ay, v));
            }
            for (int q = 1; q < k; ++q)
                for (int r = q; r > 0 && key[r] > key[r - 1]; --r) {
                    std::swap(key[r], key[r - 1]);
                    std::swap(pts[r], pts[r - 1]);
                }
        }
        pts.push_back(c);
        counts[i] = k;
        for (int q = 0; q < MAXP; ++q) {
            const V3 p = q <= k ? pts[q] : mk(0.0f, 0.0f, 0.0f);
            verts[3 * (MAXP * i + q) + 0] = p.x;
            verts[3 * (MAXP * i + q) + 1] = p.y;
            verts[3 * (MAXP * i + q) + 2] = p.z;
        }
        for (int q = 0; q < MAXP - 1; ++q) {
            int* tr = tris + 3 * ((MAXP - 1) * i + q);
            if (k >= 3 && q < k) {
                tr[0] = MAXP * i + k;
                tr[1] = MAXP * i + q;
                tr[2] = MAXP * i + (q + 1 < k ? q + 1 : 0);
            } else {
                tr[0] = tr[1] = tr[2] = -1;
            }
        }
    }
    return 0;
}

// Half conversion of the restatement, exposed for tests: n values.
void orc_round_half(const float* in, float* out, int n) {
    for (int i = 0; i < n; ++i) out[i] = h16(in[i]);
}

}  // extern "C"
