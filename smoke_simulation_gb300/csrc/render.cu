// Headless half-angle slice renderer (smk_render): the reference's two-pass volume drawing
// restated as two CUDA kernels.
//
// The reference (project/main.cpp:369-419, 474-476) draws proxy plane i into the eye buffer
// using the light buffer as it stands after planes 0..i-1, then draws the same plane into the
// light buffer.  The light buffer after plane k therefore only depends on the light's own rays,
// so it is computed for every plane first, in parallel over light texels (k_render_light: each
// texel marches the planes and stores its RGBA after each one), and the eye buffer is then
// computed in parallel over pixels (k_render_eye: each pixel marches the planes in drawing
// order, reading the light buffer of the previous plane).  Two launches per frame, no
// dependence between pixels.
//
// Per fragment (texVolume.frag:27-52, light.frag:16-23): the plane point is where the pixel's
// ray meets the plane (what rasterising the plane-box polygon and interpolating its world
// position yields), kept when it lies in the box and between the near and far planes; density
// from the 3D texture (linear filtering, clamp to edge, texel centres at (i + 0.5) / n, the
// shader's coordinate ((p - box) / (n / 2) + 1) / 2 with integer n / 2); the light colour from
// the light buffer at the point's light-projected position (linear filtering, repeat: the
// framebuffer texture's default wrap).  Eye colour = light colour, alpha = density; front-to-back
// premultiplies and blends (ONE_MINUS_DST_ALPHA, ONE), back-to-front blends (SRC_ALPHA,
// ONE_MINUS_SRC_ALPHA) with alpha (ONE, ONE_MINUS_SRC_ALPHA); the light buffer blends (0,0,0,d)
// with (SRC_ALPHA, ONE_MINUS_SRC_ALPHA) / (ONE, ONE_MINUS_SRC_ALPHA).  Every stored value is
// rounded to half precision (RGBA16F framebuffers, labhelper/fbo.cpp:46).  Weights are float
// (the GL texture unit's fixed-point weights are not reproduced).
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <string>

#include "../../include/smoke_gb300.h"
#include "common.cuh"
#include "sim_internal.h"

namespace smk {

namespace {

struct V3 {
    float x, y, z;
};
__host__ __device__ inline V3 mk(float x, float y, float z) { return V3{x, y, z}; }
__host__ __device__ inline V3 operator+(V3 a, V3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
__host__ __device__ inline V3 operator-(V3 a, V3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
__host__ __device__ inline V3 operator*(V3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
__host__ __device__ inline float dot3(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ inline V3 cross3(V3 a, V3 b) {
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline V3 norm3(V3 a) { return a * (1.0f / sqrtf(dot3(a, a))); }

// A perspective view (the camera or the light): origin, orthonormal basis as lookAt builds it,
// and the NDC scales (aspect * tan(fovy / 2), tan(fovy / 2)).
struct ViewSetup {
    V3 eye, s, u, f;
    float sx, sy, znear, zfar;
    int w, h;
};

struct Setup {
    ViewSetup cam, light;
    V3 start, end, n;  // planes: start + (end - start) * (i + 0.5) / planes, normal n
    int planes;
    int back_to_front;
    V3 box_min, box_max, box_pos, tex_half;
    float clear[4];  // the light buffer's clear colour (half-rounded)
    float bg[3];
};

ViewSetup make_view(V3 eye, V3 dir, V3 up, float fovy_deg, float aspect, float zn, float zf, int w, int h) {
    ViewSetup v;
    v.eye = eye;
    v.f = norm3(dir);
    v.s = norm3(cross3(v.f, up));
    v.u = cross3(v.s, v.f);
    const float th = (float)tan(0.5 * (double)fovy_deg * 3.14159265358979323846 / 180.0);
    v.sx = aspect * th;
    v.sy = th;
    v.znear = zn;
    v.zfar = zf;
    v.w = w;
    v.h = h;
    return v;
}

// Round-to-nearest-even to half precision and back (the value an RGBA16F texel holds).
__device__ __forceinline__ float h16(float x) { return __half2float(__float2half_rn(x)); }

Setup make_setup(const smk_render_params& rp, int nx, int ny, int nz) {
    Setup S;
    const V3 cam = mk(rp.camera_pos[0], rp.camera_pos[1], rp.camera_pos[2]);
    const V3 up = mk(rp.up[0], rp.up[1], rp.up[2]);
    const V3 lp = mk(rp.light_pos[0], rp.light_pos[1], rp.light_pos[2]);
    const V3 box = mk(rp.box_pos[0], rp.box_pos[1], rp.box_pos[2]);
    S.cam = make_view(cam, mk(rp.camera_dir[0], rp.camera_dir[1], rp.camera_dir[2]), up, rp.fovy_deg,
                      (float)rp.width / (float)rp.height, rp.znear, rp.zfar, rp.width, rp.height);
    S.light = make_view(lp, box - lp, up, rp.light_fovy_deg, 1.0f, rp.light_znear, rp.light_zfar, rp.light_res,
                        rp.light_res);
    // half vector and drawing order (main.cpp:660-661, 676-687)
    const V3 cam_view = box - cam, light_view = box - lp;
    const V3 cn = norm3(cam_view), ln = norm3(light_view);
    V3 half = cn + ln;
    if (dot3(cn, ln) < 0.0f) half = mk(-cn.x, -cn.y, -cn.z) + ln;
    S.back_to_front = dot3(cam_view, light_view) < 0.0f ? 1 : 0;
    // planes between the box corners' extreme projections on the half vector, measured from the
    // world origin with the corners at +-dimensions / 2 (boundingBox.cpp:135-181)
    const V3 dims = mk(rp.cell_size * nx, rp.cell_size * ny, rp.cell_size * nz);
    const V3 hd = dims * 0.5f;
    S.n = norm3(half);
    float mn = 0.0f, mx = 0.0f;
    for (int c = 0; c < 8; ++c) {
        const V3 corner = mk((c & 1) ? hd.x : -hd.x, (c & 2) ? hd.y : -hd.y, (c & 4) ? hd.z : -hd.z);
        const float d = dot3(corner, S.n);
        if (c == 0 || d < mn) mn = d;
        if (c == 0 || d > mx) mx = d;
    }
    S.start = S.n * mn;
    S.end = S.n * mx;
    S.planes = rp.planes;
    S.box_pos = box;
    S.box_min = box - hd;
    S.box_max = box + hd;
    S.tex_half = mk((float)(nx / 2), (float)(ny / 2), (float)(nz / 2));
    for (int k = 0; k < 3; ++k) {
        S.clear[k] = __half2float(__float2half_rn(rp.light_color[k]));
        S.bg[k] = rp.bg_color[k];
    }
    S.clear[3] = 1.0f;
    return S;
}

__device__ __forceinline__ bool inside(const Setup& S, V3 p) {
    return p.x >= S.box_min.x && p.x <= S.box_max.x && p.y >= S.box_min.y && p.y <= S.box_max.y &&
           p.z >= S.box_min.z && p.z <= S.box_max.z;
}

// The point where the ray of pixel (px, py) of view V meets plane i, if it is drawn there.
__device__ __forceinline__ bool plane_hit(const Setup& S, const ViewSetup& V, V3 d, float denom, int i, V3* p) {
    if (denom == 0.0f) return false;
    const float ti = ((float)i + 0.5f) / (float)S.planes;
    const V3 pp = S.start + (S.end - S.start) * ti;
    const float t = dot3(pp - V.eye, S.n) / denom;
    if (!(t >= V.znear && t <= V.zfar)) return false;
    *p = V.eye + d * t;
    return inside(S, *p);
}

__device__ __forceinline__ V3 ray_dir(const ViewSetup& V, int px, int py) {
    const float nx = (2.0f * ((float)px + 0.5f)) / (float)V.w - 1.0f;
    const float ny = (2.0f * ((float)py + 0.5f)) / (float)V.h - 1.0f;
    return (V.f + V.s * (nx * V.sx)) + V.u * (ny * V.sy);
}

template <typename T>
__device__ __forceinline__ float cell(const T* rho, const Grid& g, int x, int y, int z) {
    return ldv(rho, g.idx(x, y, z));
}

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// texture(gridTex, ((p - box) / (n / 2) + 1) / 2).r with linear filtering and clamp to edge
template <typename T>
__device__ float sample_density(const Setup& S, const T* rho, const Grid& g, V3 p) {
    const float tx = ((p.x - S.box_pos.x) / S.tex_half.x + 1.0f) / 2.0f;
    const float ty = ((p.y - S.box_pos.y) / S.tex_half.y + 1.0f) / 2.0f;
    const float tz = ((p.z - S.box_pos.z) / S.tex_half.z + 1.0f) / 2.0f;
    const float ux = tx * (float)g.nx - 0.5f, uy = ty * (float)g.ny - 0.5f, uz = tz * (float)g.nz - 0.5f;
    const float fx = floorf(ux), fy = floorf(uy), fz = floorf(uz);
    const float ax = ux - fx, ay = uy - fy, az = uz - fz;
    const int x0 = clampi((int)fx, 0, g.nx - 1), x1 = clampi((int)fx + 1, 0, g.nx - 1);
    const int y0 = clampi((int)fy, 0, g.ny - 1), y1 = clampi((int)fy + 1, 0, g.ny - 1);
    const int z0 = clampi((int)fz, 0, g.nz - 1), z1 = clampi((int)fz + 1, 0, g.nz - 1);
    const float c00 = cell(rho, g, x0, y0, z0) * (1.0f - ax) + cell(rho, g, x1, y0, z0) * ax;
    const float c10 = cell(rho, g, x0, y1, z0) * (1.0f - ax) + cell(rho, g, x1, y1, z0) * ax;
    const float c01 = cell(rho, g, x0, y0, z1) * (1.0f - ax) + cell(rho, g, x1, y0, z1) * ax;
    const float c11 = cell(rho, g, x0, y1, z1) * (1.0f - ax) + cell(rho, g, x1, y1, z1) * ax;
    const float c0 = c00 * (1.0f - ay) + c10 * ay;
    const float c1 = c01 * (1.0f - ay) + c11 * ay;
    return c0 * (1.0f - az) + c1 * az;
}

__device__ __forceinline__ int wrapi(int v, int n) {
    const int r = v % n;
    return r < 0 ? r + n : r;
}

// texture(lightMap, uv) of one plane's light buffer: linear filtering, repeat
__device__ float4 sample_light(const __half* L, int R, float u, float v) {
    const float sx = fminf(fmaxf(u * (float)R - 0.5f, -1.0e6f), 1.0e6f);
    const float sy = fminf(fmaxf(v * (float)R - 0.5f, -1.0e6f), 1.0e6f);
    const float fx = floorf(sx), fy = floorf(sy);
    const float ax = sx - fx, ay = sy - fy;
    const int x0 = wrapi((int)fx, R), x1 = wrapi((int)fx + 1, R);
    const int y0 = wrapi((int)fy, R), y1 = wrapi((int)fy + 1, R);
    float out[4];
    for (int c = 0; c < 4; ++c) {
        const float t00 = __half2float(L[4 * (x0 + R * y0) + c]), t10 = __half2float(L[4 * (x1 + R * y0) + c]);
        const float t01 = __half2float(L[4 * (x0 + R * y1) + c]), t11 = __half2float(L[4 * (x1 + R * y1) + c]);
        out[c] = (t00 * (1.0f - ax) + t10 * ax) * (1.0f - ay) + (t01 * (1.0f - ax) + t11 * ax) * ay;
    }
    return make_float4(out[0], out[1], out[2], out[3]);
}

// The light buffer after every plane: slices[i] = RGBA16F light buffer after drawing plane i.
template <typename T>
__global__ void k_render_light(const Setup S, const T* __restrict__ rho, const Grid g, __half* __restrict__ slices) {
    const int R = S.light.w;
    const int id = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (id >= R * R) return;
    const int lx = id % R, ly = id / R;
    const V3 d = ray_dir(S.light, lx, ly);
    const float denom = dot3(d, S.n);
    float c[4] = {S.clear[0], S.clear[1], S.clear[2], S.clear[3]};
    const size_t plane_stride = (size_t)R * R * 4;
    for (int i = 0; i < S.planes; ++i) {
        V3 p;
        if (plane_hit(S, S.light, d, denom, i, &p)) {
            const float a = sample_density(S, rho, g, p);
            const float om = 1.0f - a;
            c[0] = h16(c[0] * om);
            c[1] = h16(c[1] * om);
            c[2] = h16(c[2] * om);
            c[3] = h16(a + c[3] * om);
        }
        __half* o = slices + plane_stride * i + 4 * (size_t)id;
        o[0] = __float2half_rn(c[0]);
        o[1] = __float2half_rn(c[1]);
        o[2] = __float2half_rn(c[2]);
        o[3] = __float2half_rn(c[3]);
    }
}

template <typename T>
__global__ void k_render_eye(const Setup S, const T* __restrict__ rho, const Grid g,
                             const __half* __restrict__ slices, float* __restrict__ eye, float* __restrict__ comp) {
    const int W = S.cam.w, H = S.cam.h, R = S.light.w;
    const int id = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (id >= W * H) return;
    const int px = id % W, py = id / W;
    const V3 d = ray_dir(S.cam, px, py);
    const float denom = dot3(d, S.n);
    float e[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    const size_t plane_stride = (size_t)R * R * 4;
    for (int i = 0; i < S.planes; ++i) {
        V3 p;
        if (!plane_hit(S, S.cam, d, denom, i, &p)) continue;
        const float a = sample_density(S, rho, g, p);
        float4 lc = make_float4(S.clear[0], S.clear[1], S.clear[2], S.clear[3]);
        if (i > 0) {
            // light-projected position: NDC of the light view, mapped to [0, 1]
            const V3 q = p - S.light.eye;
            const float depth = dot3(q, S.light.f);
            const float u = (dot3(q, S.light.s) / (S.light.sx * depth)) * 0.5f + 0.5f;
            const float v = (dot3(q, S.light.u) / (S.light.sy * depth)) * 0.5f + 0.5f;
            lc = sample_light(slices + plane_stride * (i - 1), R, u, v);
        }
        if (S.back_to_front) {
            const float om = 1.0f - a;
            e[0] = h16(lc.x * a + e[0] * om);
            e[1] = h16(lc.y * a + e[1] * om);
            e[2] = h16(lc.z * a + e[2] * om);
            e[3] = h16(a + e[3] * om);
        } else {
            const float om = 1.0f - e[3];
            e[0] = h16((lc.x * a) * om + e[0]);
            e[1] = h16((lc.y * a) * om + e[1]);
            e[2] = h16((lc.z * a) * om + e[2]);
            e[3] = h16(a * om + e[3]);
        }
    }
    float* o = eye + 4 * (size_t)id;
    o[0] = e[0];
    o[1] = e[1];
    o[2] = e[2];
    o[3] = e[3];
    if (comp) {
        float* c = comp + 3 * (size_t)id;
        const float om = 1.0f - e[3];
        c[0] = e[0] * e[3] + S.bg[0] * om;
        c[1] = e[1] * e[3] + S.bg[1] * om;
        c[2] = e[2] * e[3] + S.bg[2] * om;
    }
}

}  // namespace
}  // namespace smk

using namespace smk;

extern "C" {

void smk_default_render_params(smk_render_params* rp) {
    if (!rp) return;
    *rp = smk_render_params{};
    rp->width = 1280;
    rp->height = 720;
    rp->light_res = 512;
    rp->planes = 100;
    const float cam[3] = {1.0f, 20.0f, 100.0f};
    const float len = sqrtf(cam[0] * cam[0] + cam[1] * cam[1] + cam[2] * cam[2]);
    for (int k = 0; k < 3; ++k) {
        rp->camera_pos[k] = cam[k];
        rp->camera_dir[k] = -cam[k] * (1.0f / len);
    }
    rp->up[1] = 1.0f;
    rp->fovy_deg = 45.0f;
    rp->znear = 5.0f;
    rp->zfar = 2000.0f;
    rp->light_pos[0] = 120.0f;
    rp->light_pos[1] = 80.0f;
    rp->light_fovy_deg = 45.0f;
    rp->light_znear = 5.0f;
    rp->light_zfar = 2000.0f;
    rp->light_color[0] = 0.9882f;
    rp->light_color[1] = 0.9333f;
    rp->light_color[2] = 0.7549f;
    rp->cell_size = 1.0f;
    for (int k = 0; k < 3; ++k) rp->bg_color[k] = 20.0f / 255.0f;
}

int smk_render(smk_sim* sim, const smk_render_params* rp, float* eye_rgba, float* composite_rgb, void* stream) {
    if (!sim || !rp || !eye_rgba) return smk_fail(SMK_ERR_INVALID, "null argument");
    if (rp->width < 1 || rp->height < 1 || rp->light_res < 1 || rp->planes < 1 || rp->planes > 100000 ||
        (long long)rp->width * rp->height > (1LL << 28) || rp->light_res > 16384 || !(rp->cell_size > 0.0f))
        return smk_fail(SMK_ERR_INVALID, "invalid render parameters");
    if (sim->g.nx < 2 || sim->g.ny < 2 || sim->g.nz < 2)
        return smk_fail(SMK_ERR_INVALID, "the renderer needs at least 2 cells per axis");
    DeviceGuard dg(sim->device);
    cudaStream_t st = (cudaStream_t)stream;
    const size_t need = (size_t)rp->planes * rp->light_res * rp->light_res * 4 * sizeof(__half);
    if (sim->render_scratch_bytes < need) {
        if (sim->render_scratch) cudaFree(sim->render_scratch);
        sim->render_scratch = nullptr;
        sim->render_scratch_bytes = 0;
        SMK_CUDA(cudaMalloc(&sim->render_scratch, need));
        sim->render_scratch_bytes = need;
    }
    const Setup S = make_setup(*rp, sim->g.nx, sim->g.ny, sim->g.nz);
    __half* slices = static_cast<__half*>(sim->render_scratch);
    const float* rho = sim->rho[sim->index_now ^ 1];
    const int R2 = rp->light_res * rp->light_res, WH = rp->width * rp->height;
    if (sim->rho_bf16) {
        const __nv_bfloat16* r = reinterpret_cast<const __nv_bfloat16*>(rho);
        k_render_light<<<(R2 + 255) / 256, 256, 0, st>>>(S, r, sim->g, slices);
        k_render_eye<<<(WH + 255) / 256, 256, 0, st>>>(S, r, sim->g, slices, eye_rgba, composite_rgb);
    } else {
        k_render_light<<<(R2 + 255) / 256, 256, 0, st>>>(S, rho, sim->g, slices);
        k_render_eye<<<(WH + 255) / 256, 256, 0, st>>>(S, rho, sim->g, slices, eye_rgba, composite_rgb);
    }
    SMK_CUDA(cudaGetLastError());
    return SMK_OK;
}

}  // extern "C"
