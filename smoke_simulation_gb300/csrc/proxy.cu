// Proxy-slice geometry on the device (smk_proxy_planes): the polygons of the reference's
// half-angle proxy planes (project/boundingBox.cpp:133-181 generateProxyGeometry, 87-92
// pseudoangle, 231-360 getMinMaxPoints / teselate / sortPoints / rayPlaneIntersection /
// planeBoxIntersections / duplicate), one thread per plane, for callers that still draw the
// planes with a graphics API (the headless renderer in render.cu intersects rays with the
// planes directly and needs no polygons).
//
// Every float operation follows the reference's order, so the result is bit for bit the
// reference's (the reference's own functions, built for the host, are the checker): the ray
// direction d1 = normalize(-view_dir), normalised once more (d2) where getMinMaxPoints and
// sortPoints normalise their argument; start/end = view_origin + d1 * (the extreme projections
// on d2 of the box corners +-dims/2 about the world origin); plane i at start + (end - start) *
// ((i + 0.5) / P) with normal d1; its polygon: the intersections of the plane with the box's 12
// edges (each a ray from a corner along an axis, parameter in [0, edge length]), exact repeats
// dropped, the centroid (sum / count) appended; the points sorted by pseudo-angle about the
// centroid in the plane basis (ax = normalize(p0 - centroid), ay = cross(d2, ax)), descending,
// with the reference's double-precision literals (1. + r, 3. - r); a fan around the centroid.
// One deviation: an edge lying in the plane (0 / 0) yields no point, where the reference keeps a
// NaN point.
#include <cuda_runtime.h>
#include <math.h>

#include "../../include/smoke_gb300.h"
#include "sim_internal.h"

namespace smk {
namespace {

struct P3 {
    float x, y, z;
};
__host__ __device__ inline P3 pk(float x, float y, float z) { return P3{x, y, z}; }
__host__ __device__ inline P3 padd(P3 a, P3 b) { return pk(a.x + b.x, a.y + b.y, a.z + b.z); }
__host__ __device__ inline P3 psub(P3 a, P3 b) { return pk(a.x - b.x, a.y - b.y, a.z - b.z); }
__host__ __device__ inline P3 pscl(P3 a, float s) { return pk(a.x * s, a.y * s, a.z * s); }
__host__ __device__ inline float pdot(P3 a, P3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ inline P3 pcross(P3 a, P3 b) {
    return pk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__host__ __device__ inline P3 pnorm(P3 a) { return pscl(a, 1.0f / sqrtf(pdot(a, a))); }

// pseudoangle (boundingBox.cpp:87-92): its literals are doubles, so 1. + r and 3. - r are
// evaluated in double and rounded to the float result
__device__ inline float pseudoangle(float y, float x) {
    const float r = x / (fabsf(x) + fabsf(y));
    if (y < 0.0f) return (float)(1.0 + (double)r);
    return (float)(3.0 - (double)r);
}

struct ProxySetup {
    P3 start, end, d, d2, box, half, dims;
    int planes;
};

constexpr int MAXP = 7;  // at most 6 polygon points + the centroid

__global__ void k_proxy_planes(const ProxySetup S, float* __restrict__ verts, int* __restrict__ counts,
                               int* __restrict__ tris) {
    const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (i >= S.planes) return;
    const float t = ((float)i + 0.5f) / (float)S.planes;
    const P3 o = padd(S.start, pscl(psub(S.end, S.start), t));
    P3 pts[MAXP];
    int k = 0;
    P3 c = pk(0.0f, 0.0f, 0.0f);
    // edges along x, y, z: from box - half*(1, sy, sz) etc. (planeBoxIntersections order)
    for (int axis = 0; axis < 3; ++axis)
        for (int a = -1; a < 2; a += 2)
            for (int b = -1; b < 2; b += 2) {
                P3 ro, rd;
                float len;
                if (axis == 0) {
                    ro = psub(S.box, pk(S.half.x, S.half.y * (float)a, S.half.z * (float)b));
                    rd = pk(1.0f, 0.0f, 0.0f);
                    len = S.dims.x;
                } else if (axis == 1) {
                    ro = psub(S.box, pk(S.half.x * (float)a, S.half.y, S.half.z * (float)b));
                    rd = pk(0.0f, 1.0f, 0.0f);
                    len = S.dims.y;
                } else {
                    ro = psub(S.box, pk(S.half.x * (float)b, S.half.y * (float)a, S.half.z));
                    rd = pk(0.0f, 0.0f, 1.0f);
                    len = S.dims.z;
                }
                const float den = pdot(rd, S.d);
                if (den == 0.0f) continue;
                const float tt = pdot(psub(o, ro), S.d) / den;
                if (tt > len || tt < 0.0f) continue;
                const P3 p = padd(ro, pscl(rd, tt));
                bool dup = false;
                for (int q = 0; q < k; ++q) dup = dup || (p.x == pts[q].x && p.y == pts[q].y && p.z == pts[q].z);
                if (!dup && k < MAXP - 1) {
                    pts[k++] = p;
                    c = padd(c, p);
                }
            }
    if (k > 0) c = pk(c.x / (float)k, c.y / (float)k, c.z / (float)k);
    // sort the k points by pseudo-angle about the centroid, descending (insertion sort; keys of a
    // convex polygon's vertices are distinct)
    if (k > 0) {
        const P3 ax = pnorm(psub(pts[0], c));
        const P3 ay = pcross(S.d2, ax);
        float key[MAXP];
        for (int q = 0; q < k; ++q) {
            const P3 v = psub(pts[q], c);
            key[q] = pseudoangle(pdot(ay, v), pdot(ax, v));
        }
        for (int q = 1; q < k; ++q)
            for (int r = q; r > 0 && key[r] > key[r - 1]; --r) {
                const float tk = key[r];
                key[r] = key[r - 1];
                key[r - 1] = tk;
                const P3 tp = pts[r];
                pts[r] = pts[r - 1];
                pts[r - 1] = tp;
            }
    }
    pts[k] = c;
    counts[i] = k;
    for (int q = 0; q < MAXP; ++q) {
        const P3 p = q <= k ? pts[q] : pk(0.0f, 0.0f, 0.0f);
        verts[3 * (MAXP * i + q) + 0] = p.x;
        verts[3 * (MAXP * i + q) + 1] = p.y;
        verts[3 * (MAXP * i + q) + 2] = p.z;
    }
    // fan around the centroid (local vertex k): (k, q, q+1) for q < k-1, then (k, k-1, 0)
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

}  // namespace
}  // namespace smk

using namespace smk;

extern "C" {

int smk_proxy_planes(const float view_origin[3], const float view_dir[3], const float box_pos[3],
                     const float dims[3], int planes, float* vertices, int* counts, int* triangles, void* stream) {
    if (!view_origin || !view_dir || !box_pos || !dims || !vertices || !counts || !triangles || planes < 1)
        return smk_fail(SMK_ERR_INVALID, "invalid proxy-plane arguments");
    ProxySetup S;
    S.d = pnorm(pk(-view_dir[0], -view_dir[1], -view_dir[2]));
    S.d2 = pnorm(S.d);
    S.box = pk(box_pos[0], box_pos[1], box_pos[2]);
    S.dims = pk(dims[0], dims[1], dims[2]);
    S.half = pk(S.dims.x / 2.0f, S.dims.y / 2.0f, S.dims.z / 2.0f);
    const P3 vo = pk(view_origin[0], view_origin[1], view_origin[2]);
    // the corners as generateProxyGeometry lists them (vec3(+-1, +-1, +-1) * dims / 2)
    static const float corner_sign[8][3] = {{-1, -1, 1}, {1, -1, 1}, {-1, 1, 1}, {1, 1, 1},
                                            {-1, -1, -1}, {1, -1, -1}, {-1, 1, -1}, {1, 1, -1}};
    float mn = 0.0f, mx = 0.0f;
    for (int c = 0; c < 8; ++c) {
        const P3 corner = pk(corner_sign[c][0] * S.dims.x / 2.0f, corner_sign[c][1] * S.dims.y / 2.0f,
                             corner_sign[c][2] * S.dims.z / 2.0f);
        const float dd = pdot(psub(corner, vo), S.d2);
        if (c == 0) mn = mx = dd;
        if (dd < mn) mn = dd;
        if (dd > mx) mx = dd;
    }
    S.start = padd(vo, pscl(S.d, mn));
    S.end = padd(vo, pscl(S.d, mx));
    S.planes = planes;
    k_proxy_planes<<<(planes + 127) / 128, 128, 0, (cudaStream_t)stream>>>(S, vertices, counts, triangles);
    SMK_CUDA(cudaGetLastError());
    return SMK_OK;
}

}  // extern "C"
