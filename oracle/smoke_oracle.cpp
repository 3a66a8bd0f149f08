// TEST INFRASTRUCTURE ONLY -- the oracle.  Only tests/, __graft_entry__.smoke() and the
// cpu_baseline leg of bench.py may load this library, and only as the checker (never as the
// thing measured or shipped).  The product path (libsmoke_gb300) never links or calls it.
//
// CPU restatement of the reference's semi-Lagrangian smoke step on a staggered MAC grid
// (RasmusAlmryd/smoke-simulation, project/smokeSimulation.cu).  Every stage follows the
// reference line by line, in the reference's own memory layout:
//   cells  : n_x*n_y*n_z, index x + y*n_x + z*n_x*n_y                    (smokeSimulation.cu:127-128)
//   faces  : (n_x+1)(n_y+1)(n_z+1) for each of u, v, w, index with stride n+1 (:146-147)
//   mask s : uint8, 1 = fluid, 0 = solid                                   (:193-207, :306-309)
//
// The same code is instantiated twice:
//   T = float  : bit-faithful to the reference's arithmetic when compiled without FMA
//                contraction (-ffp-contract=off).  Sub-expressions the reference evaluates in
//                double (the over-relaxation factor, :384; the density backtrace, :628-630)
//                are evaluated in double here too.
//   T = double : the FP64 oracle of the same discretisation.  Geometry predicates (emitter and
//                obstacle rasterisation) stay in float so both instantiations see identical masks.
//
// Two projection schemes are restated:
//   velocity : the reference's in-place red-black SOR on face velocities (:356-394, :795-801).
//   pressure : the same red-black SOR written on a cell pressure P with right-hand side
//              b = -div(u*), followed by one gradient subtract.  In exact arithmetic the two
//              produce identical iterates (the reference's per-cell correction p_t accumulates
//              into P); in floating point they differ by rounding.  This is the scheme the GPU
//              library runs by default, and this restatement fixes its exact operation order
//              (fmaf where the GPU kernels use a fused multiply-add).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

extern "C" {

// Object records use the reference's own packing (smokeSimulation.cu:719-725, :750-758).
//   sphere source : x, y, z, r                         (4 floats)
//   obstacle      : x, y, z, vx, vy, vz, r             (7 floats)
//   box emitter   : x0, y0, z0, x1, y1, z1, density, vy, set_vy  (9 floats; half-open integer box)
typedef struct {
    float gravity;       // reference default -9.82  (:28)
    float buoyancy;      // reference default 2.0    (:29)
    float clamp_const;   // MAX_VELOCITY_PER_STEP 3.0 (:39)
    int clamp_mode;      // 0 reference clamp (:343-349), 1 true magnitude clamp, 2 none
    int scheme;          // 0 velocity-space SOR (reference), 1 pressure-form SOR
    int iterations;      // reference num_iterations 30 (:797); for scheme 1 the sweep cap
    double omega;        // OVER_RELAXATION 1.9 (:38)
    float tol;           // scheme 1: stop on max|residual| <= tol (0 disables)
    int check_every;     // scheme 1: residual check cadence in sweeps
    int warm_start;      // scheme 1: keep P across steps
    const float* spheres;   int n_spheres;
    const float* boxes;     int n_boxes;
    const float* obstacles; int n_obstacles;
    int refine;          // scheme 1 with tol > 0: FP64-checked refinement rounds (0: none)
    int refine_sweeps;   // sweeps of each correction solve
    int obstacle_velocity;  // 1: faces touching a cell of the last obstacle take its velocity
    int solver;          // scheme 1: 0 red-black SOR, 1 weighted Jacobi (weight omega)
} orc_params;

typedef struct {
    int nx, ny, nz;
    void* rho[2];
    void* u[2];
    void* v[2];
    void* w[2];
    uint8_t* s;
    void* P;        // scheme 1 only (cells), may be null for scheme 0
    void* b;        // scheme 1 only (cells)
    int index_now;  // the reference's indexNow (:707); 1 before the first step
} orc_state;

typedef struct {
    int sweeps;         // sweeps performed in the projection
    int converged;      // scheme 1 with tol > 0: the tolerance rule ended the solve
    float resid_max;    // scheme 1: max |residual| at the last check (or final state)
    float div_max;      // max |div u| over projectable cells after projection
    int refine_rounds;  // correction rounds applied (refine > 0)
    float div64_max;    // max |div u| of the last FP64 measurement (refine > 0), else -1
} orc_stats;

}  // extern "C"

namespace {

struct Dims {
    int nx, ny, nz;
    inline long long c(int x, int y, int z) const {
        return (long long)x + (long long)y * nx + (long long)z * nx * ny;
    }
    inline long long f(int x, int y, int z) const {
        return (long long)x + (long long)y * (nx + 1) + (long long)z * (nx + 1) * (ny + 1);
    }
    long long ncells() const { return (long long)nx * ny * nz; }
    long long nfaces() const { return (long long)(nx + 1) * (ny + 1) * (nz + 1); }
};

// ---- stage a4: emitters and obstacles (smokeSimulation.cu:251-273, :289-313) ----------------

// Box emitters: the reference has no box source; its documented emulation writes density into
// both ping-pong buffers before simulate() (equivalent to fillSmoke, which runs first).  The
// optional upward velocity goes to the v-faces below and above each box cell in buffer "now".
template <typename T>
void emit_boxes(const Dims& d, T* rho0, T* rho1, T* v_now, const float* boxes, int nb) {
    for (int i = 0; i < nb; ++i) {
        const float* bx = boxes + 9 * i;
        int x0 = std::max(0, (int)bx[0]), y0 = std::max(0, (int)bx[1]), z0 = std::max(0, (int)bx[2]);
        int x1 = std::min(d.nx, (int)bx[3]), y1 = std::min(d.ny, (int)bx[4]), z1 = std::min(d.nz, (int)bx[5]);
        T dens = (T)bx[6];
        for (int z = z0; z < z1; ++z)
            for (int y = y0; y < y1; ++y)
                for (int x = x0; x < x1; ++x) {
                    rho0[d.c(x, y, z)] = dens;
                    rho1[d.c(x, y, z)] = dens;
                    if (bx[8] != 0.0f && v_now) {
                        v_now[d.f(x, y, z)] = (T)bx[7];
                        v_now[d.f(x, y + 1, z)] = (T)bx[7];
                    }
                }
    }
}

// fillSmoke (:251-273): interior cells [1, n-2]; squared distance in float from the integer
// cell corner; both buffers set to 1.  powf(d, 2) is written d*d (exact for the integer and
// half-integer geometry used by every scene here).
template <typename T>
void fill_smoke(const Dims& d, T* rho0, T* rho1, const float* sp, int ns) {
#pragma omp parallel for schedule(static)
    for (int z = 1; z < d.nz - 1; ++z)
        for (int y = 1; y < d.ny - 1; ++y)
            for (int x = 1; x < d.nx - 1; ++x)
                for (int i = 0; i < ns; ++i) {
                    float dx = (float)x - sp[4 * i + 0];
                    float dy = (float)y - sp[4 * i + 1];
                    float dz = (float)z - sp[4 * i + 2];
                    float sr = sp[4 * i + 3];
                    float dist = dx * dx + dy * dy + dz * dz;
                    if (dist < sr * sr) {
                        rho0[d.c(x, y, z)] = (T)1.0f;
                        rho1[d.c(x, y, z)] = (T)1.0f;
                    }
                }
}

// fillObstacle (:289-313): interior cells, every obstacle overwrites the cell (last one wins).
void fill_obstacles(const Dims& d, uint8_t* s, const float* ob, int no) {
#pragma omp parallel for schedule(static)
    for (int z = 1; z < d.nz - 1; ++z)
        for (int y = 1; y < d.ny - 1; ++y)
            for (int x = 1; x < d.nx - 1; ++x)
                for (int i = 0; i < no; ++i) {
                    float dx = (float)x - ob[7 * i + 0];
                    float dy = (float)y - ob[7 * i + 1];
                    float dz = (float)z - ob[7 * i + 2];
                    float sr = ob[7 * i + 6];
                    float dist = dx * dx + dy * dy + dz * dz;
                    s[d.c(x, y, z)] = (dist < sr * sr) ? 0 : 1;
                }
}

// ---- stage b: forcing (a5, :315-329) + velocity clamp (a6, :331-352) -------------------------

template <typename T>
void forcing(const Dims& d, T* u, T* v, T* w, const T* rho, const uint8_t* s, float dt, float g,
             float alpha, float clamp_const, int clamp_mode) {
    const T tdt = (T)dt, tg = (T)g, ta = (T)alpha;
    // integrate: x,z in [0,n), y in [1,n); both cells of the v-face fluid.
#pragma omp parallel for schedule(static)
    for (int z = 0; z < d.nz; ++z)
        for (int y = 1; y < d.ny; ++y)
            for (int x = 0; x < d.nx; ++x) {
                if (s[d.c(x, y, z)] != 0 && s[d.c(x, y - 1, z)] != 0) {
                    T r = rho[d.c(x, y, z)];
                    T buoy = ta * (r - (T)0.0f);
                    T add = r * tg * tdt + buoy * tdt;
                    v[d.f(x, y, z)] = v[d.f(x, y, z)] + add;
                }
            }
    if (clamp_mode == 2) return;
    // velocityConfinement: x,y,z in [1,n) at the shared staggered index.
    const float lim_sq_f = clamp_const * clamp_const;  // MAX*MAX in float (:345)
#pragma omp parallel for schedule(static)
    for (int z = 1; z < d.nz; ++z)
        for (int y = 1; y < d.ny; ++y)
            for (int x = 1; x < d.nx; ++x) {
                long long i = d.f(x, y, z);
                T ut = u[i], vt = v[i], wt = w[i];
                T len = ut * ut + vt * vt + wt * wt;
                if (clamp_mode == 0) {
                    if (len * tdt > (T)lim_sq_f) {
                        T f = (T)lim_sq_f / (len * tdt);
                        u[i] = ut * f;
                        v[i] = vt * f;
                        w[i] = wt * f;
                    }
                } else {
                    // true magnitude clamp |u| <= clamp_const
                    T lim = (T)clamp_const;
                    if (len > lim * lim) {
                        T f = lim / std::sqrt(len);
                        u[i] = ut * f;
                        v[i] = vt * f;
                        w[i] = wt * f;
                    }
                }
            }
}

// ---- stage c/d: projection ------------------------------------------------------------------

// Reference velocity-space red-black SOR (:356-394), colour k = cells with (x+y+z+k) even.
template <typename T>
void project_velocity(const Dims& d, T* u, T* v, T* w, const uint8_t* s, int iters, double omega) {
    for (int it = 0; it < iters; ++it)
        for (int colour = 0; colour < 2; ++colour) {
#pragma omp parallel for schedule(static)
            for (int z = 1; z < d.nz - 1; ++z)
                for (int y = 1; y < d.ny - 1; ++y) {
                    int xs = 1 + ((1 + y + z + colour) & 1);
                    for (int x = xs; x < d.nx - 1; x += 2) {
                        if (s[d.c(x, y, z)] == 0) continue;
                        int sx1 = s[d.c(x + 1, y, z)], sx0 = s[d.c(x - 1, y, z)];
                        int sy1 = s[d.c(x, y + 1, z)], sy0 = s[d.c(x, y - 1, z)];
                        int sz1 = s[d.c(x, y, z + 1)], sz0 = s[d.c(x, y, z - 1)];
                        int acc = sx0 + sx1 + sy0 + sy1 + sz0 + sz1;
                        if (acc == 0) continue;
                        long long i = d.f(x, y, z);
                        long long ix = d.f(x + 1, y, z), iy = d.f(x, y + 1, z), iz = d.f(x, y, z + 1);
                        T div = -u[i] + u[ix] + -v[i] + v[iy] + -w[i] + w[iz];
                        T pt;
                        if (sizeof(T) == sizeof(float)) {
                            float q = (float)(-div) / (float)acc;
                            pt = (T)(float)((double)q * omega);
                        } else {
                            pt = (T)((-div / (T)acc) * (T)omega);
                        }
                        u[i] -= pt * (T)sx0;
                        u[ix] += pt * (T)sx1;
                        v[i] -= pt * (T)sy0;
                        v[iy] += pt * (T)sy1;
                        w[i] -= pt * (T)sz0;
                        w[iz] += pt * (T)sz1;
                    }
                }
        }
}

inline int fluid_nbrs(const Dims& d, const uint8_t* s, int x, int y, int z) {
    return s[d.c(x + 1, y, z)] + s[d.c(x - 1, y, z)] + s[d.c(x, y + 1, z)] + s[d.c(x, y - 1, z)] +
           s[d.c(x, y, z + 1)] + s[d.c(x, y, z - 1)];
}

inline bool projectable(const Dims& d, const uint8_t* s, int x, int y, int z) {
    if (x < 1 || y < 1 || z < 1 || x > d.nx - 2 || y > d.ny - 2 || z > d.nz - 2) return false;
    if (s[d.c(x, y, z)] == 0) return false;
    return fluid_nbrs(d, s, x, y, z) > 0;
}

template <typename T>
inline T fma_t(T a, T b, T c) {
    return std::fma(a, b, c);
}

// Neighbour sum of the pressure scheme, in a fixed tree order (depth 3, so the GPU kernels'
// dependent-add chain is short): ((P_x- + P_x+) + (P_y- + P_y+)) + (P_z- + P_z+).
template <typename T>
inline T nbr_sum(const Dims& d, const T* P, int x, int y, int z) {
    const T sx = P[d.c(x - 1, y, z)] + P[d.c(x + 1, y, z)];
    const T sy = P[d.c(x, y - 1, z)] + P[d.c(x, y + 1, z)];
    const T sz = P[d.c(x, y, z - 1)] + P[d.c(x, y, z + 1)];
    return (sx + sy) + sz;
}

// max |r| as the GPU reduces it: the largest IEEE bit pattern of |r| (so NaN wins).
template <typename T>
inline void max_abs_bits(T val, T& m) {
    T a = std::fabs(val);
    if (sizeof(T) == sizeof(float)) {
        float af = (float)a, mf = (float)m;
        uint32_t ab, mb;
        std::memcpy(&ab, &af, 4);
        std::memcpy(&mb, &mf, 4);
        if (ab > mb) m = a;
    } else {
        if (!(a <= m)) m = a;
    }
}

template <typename T>
T residual_max(const Dims& d, const T* P, const T* b, const uint8_t* s) {
    T m = 0;
    for (int z = 1; z < d.nz - 1; ++z)
        for (int y = 1; y < d.ny - 1; ++y)
            for (int x = 1; x < d.nx - 1; ++x) {
                if (!projectable(d, s, x, y, z)) continue;
                int acc = fluid_nbrs(d, s, x, y, z);
                T sum = nbr_sum(d, P, x, y, z);
                T r = fma_t<T>(-(T)acc, P[d.c(x, y, z)], b[d.c(x, y, z)] + sum);
                max_abs_bits(r, m);
            }
    return m;
}

// Pressure-form red-black SOR.  rhs b = -div(u*) on projectable cells (fluid, interior, at
// least one fluid neighbour -- exactly the cells the reference updates), 0 elsewhere; P stays 0
// on every other cell, so neighbour sums need no mask.  One sweep = colour 0 then colour 1.
//   r      = fma(-acc, P_c, b_c + nbr_sum)
//   P_c   <- fma(omega/acc, r, P_c)           (omega/acc rounded to T once per acc value)
// Tolerance rule (tol > 0): at every check point j = k*check_every the residual max of the
// current state is computed, and if it is <= tol the solve ends there, on that state (sweeps =
// j).  The GPU kernels follow the same rule.
template <typename T>
int project_pressure(const Dims& d, T* u, T* v, T* w, T* P, T* b, const uint8_t* s, int max_sweeps,
                     double omega, float tol, int check_every, int warm_start, orc_stats* st,
                     int solver = 0) {
    // right-hand side
#pragma omp parallel for schedule(static)
    for (int z = 0; z < d.nz; ++z)
        for (int y = 0; y < d.ny; ++y)
            for (int x = 0; x < d.nx; ++x) {
                long long c = d.c(x, y, z);
                if (!projectable(d, s, x, y, z)) {
                    b[c] = 0;
                    P[c] = 0;
                    continue;
                }
                long long i = d.f(x, y, z);
                T div = -u[i] + u[d.f(x + 1, y, z)] + -v[i] + v[d.f(x, y + 1, z)] + -w[i] +
                        w[d.f(x, y, z + 1)];
                b[c] = -div;
                if (!warm_start) P[c] = 0;
            }
    T wacc[7];
    wacc[0] = 0;
    for (int a = 1; a <= 6; ++a) wacc[a] = (T)((T)omega / (T)a);
    if (sizeof(T) == sizeof(float)) {
        for (int a = 1; a <= 6; ++a) wacc[a] = (T)((float)omega / (float)a);
    }
    int sweeps = 0;
    int converged = 0;
    T last_r = 0;
    const int G = check_every > 0 ? check_every : 1;
    while (sweeps < max_sweeps) {
        if (tol > 0.0f && sweeps % G == 0) {
            last_r = residual_max(d, P, b, s);
            if (last_r <= (T)tol) {
                converged = 1;
                break;
            }
        }
        int group_end = (tol > 0.0f) ? std::min(max_sweeps, (sweeps / G + 1) * G) : max_sweeps;
        for (; sweeps < group_end; ++sweeps) {
            if (solver == 1) {
                // weighted Jacobi: every projectable cell from the previous iterate, the same
                // residual and update expressions as a colour pass
                std::vector<T> Pn((size_t)d.nx * d.ny * d.nz, (T)0);
#pragma omp parallel for schedule(static)
                for (int z = 1; z < d.nz - 1; ++z)
                    for (int y = 1; y < d.ny - 1; ++y)
                        for (int x = 1; x < d.nx - 1; ++x) {
                            if (!projectable(d, s, x, y, z)) continue;
                            int acc = fluid_nbrs(d, s, x, y, z);
                            long long c = d.c(x, y, z);
                            T sum = nbr_sum(d, P, x, y, z);
                            T r = fma_t<T>(-(T)acc, P[c], b[c] + sum);
                            Pn[c] = fma_t<T>(wacc[acc], r, P[c]);
                        }
#pragma omp parallel for schedule(static)
                for (int z = 1; z < d.nz - 1; ++z)
                    for (int y = 1; y < d.ny - 1; ++y)
                        for (int x = 1; x < d.nx - 1; ++x)
                            if (projectable(d, s, x, y, z)) P[d.c(x, y, z)] = Pn[d.c(x, y, z)];
                continue;
            }
            for (int colour = 0; colour < 2; ++colour) {
#pragma omp parallel for schedule(static)
                for (int z = 1; z < d.nz - 1; ++z)
                    for (int y = 1; y < d.ny - 1; ++y) {
                        int xs = 1 + ((1 + y + z + colour) & 1);
                        for (int x = xs; x < d.nx - 1; x += 2) {
                            if (!projectable(d, s, x, y, z)) continue;
                            int acc = fluid_nbrs(d, s, x, y, z);
                            long long c = d.c(x, y, z);
                            T sum = nbr_sum(d, P, x, y, z);
                            T r = fma_t<T>(-(T)acc, P[c], b[c] + sum);
                            P[c] = fma_t<T>(wacc[acc], r, P[c]);
                        }
                    }
            }
        }
    }
    // gradient subtract on faces whose two cells are both fluid (P = 0 off the projectable set)
#pragma omp parallel for schedule(static)
    for (int z = 1; z < d.nz - 1; ++z)
        for (int y = 1; y < d.ny - 1; ++y)
            for (int x = 1; x < d.nx; ++x)
                if (s[d.c(x - 1, y, z)] && s[d.c(x, y, z)]) {
                    long long i = d.f(x, y, z);
                    u[i] = u[i] - (P[d.c(x, y, z)] - P[d.c(x - 1, y, z)]);
                }
#pragma omp parallel for schedule(static)
    for (int z = 1; z < d.nz - 1; ++z)
        for (int y = 1; y < d.ny; ++y)
            for (int x = 1; x < d.nx - 1; ++x)
                if (s[d.c(x, y - 1, z)] && s[d.c(x, y, z)]) {
                    long long i = d.f(x, y, z);
                    v[i] = v[i] - (P[d.c(x, y, z)] - P[d.c(x, y - 1, z)]);
                }
#pragma omp parallel for schedule(static)
    for (int z = 1; z < d.nz; ++z)
        for (int y = 1; y < d.ny - 1; ++y)
            for (int x = 1; x < d.nx - 1; ++x)
                if (s[d.c(x, y, z - 1)] && s[d.c(x, y, z)]) {
                    long long i = d.f(x, y, z);
                    w[i] = w[i] - (P[d.c(x, y, z)] - P[d.c(x, y, z - 1)]);
                }
    if (st) {
        st->sweeps = sweeps;
        st->converged = converged;
        st->resid_max = (float)(tol > 0.0f ? last_r : 0);
    }
    return sweeps;
}

// ---- stage a: advection (a8-a10) ------------------------------------------------------------

template <typename T>
inline T avgU(const T* vel, const Dims& d, int x, int y, int z) {  // :409-420
    T s = vel[d.f(x, y, z - 1)] + vel[d.f(x + 1, y, z - 1)] + vel[d.f(x, y - 1, z - 1)] +
          vel[d.f(x + 1, y - 1, z - 1)] + vel[d.f(x, y, z)] + vel[d.f(x + 1, y, z)] +
          vel[d.f(x, y - 1, z)] + vel[d.f(x + 1, y - 1, z)];
    return s / (T)8;
}
template <typename T>
inline T avgV(const T* vel, const Dims& d, int x, int y, int z) {  // :422-434
    T s = vel[d.f(x, y, z - 1)] + vel[d.f(x - 1, y, z - 1)] + vel[d.f(x, y + 1, z - 1)] +
          vel[d.f(x - 1, y + 1, z - 1)] + vel[d.f(x, y, z)] + vel[d.f(x - 1, y, z)] +
          vel[d.f(x, y + 1, z)] + vel[d.f(x - 1, y + 1, z)];
    return s / (T)8;
}
template <typename T>
inline T avgW(const T* vel, const Dims& d, int x, int y, int z) {  // :436-447
    T s = vel[d.f(x, y, z)] + vel[d.f(x - 1, y, z)] + vel[d.f(x, y - 1, z)] +
          vel[d.f(x - 1, y - 1, z)] + vel[d.f(x, y, z - 1)] + vel[d.f(x - 1, y, z - 1)] +
          vel[d.f(x, y - 1, z - 1)] + vel[d.f(x - 1, y - 1, z - 1)];
    return s / (T)8;
}

inline float fminT(float a, float b) { return fminf(a, b); }
inline double fminT(double a, double b) { return fmin(a, b); }
inline float fmaxT(float a, float b) { return fmaxf(a, b); }
inline double fmaxT(double a, double b) { return fmax(a, b); }
inline float floorT(float a) { return floorf(a); }
inline double floorT(double a) { return floor(a); }

// sampleSmoke (:451-484): clamp to [1, n-1] with the CELL dims, trilinear with offset delta;
// `sx, sxy` are the strides of the sampled field.
template <typename T>
inline T sample(const T* f, long long sx, long long sxy, T px, T py, T pz, T dx, T dy, T dz,
                const Dims& d) {
    T x = fmaxT(fminT(px, (T)(unsigned)(d.nx - 1)), (T)1);
    T y = fmaxT(fminT(py, (T)(unsigned)(d.ny - 1)), (T)1);
    T z = fmaxT(fminT(pz, (T)(unsigned)(d.nz - 1)), (T)1);
    int x0 = (int)fminT(floorT(x - dx), (T)(unsigned)(d.nx - 1));
    T xw1 = (x - dx) - (T)x0;
    T xw0 = (T)1 - xw1;
    int x1 = (int)fminT((T)(x0 + 1), (T)(unsigned)(d.nx - 1));
    int y0 = (int)fminT(floorT(y - dy), (T)(unsigned)(d.ny - 1));
    T yw1 = (y - dy) - (T)y0;
    T yw0 = (T)1 - yw1;
    int y1 = (int)fminT((T)(y0 + 1), (T)(unsigned)(d.ny - 1));
    int z0 = (int)fminT(floorT(z - dz), (T)(unsigned)(d.nz - 1));
    T zw1 = (z - dz) - (T)z0;
    T zw0 = (T)1 - zw1;
    int z1 = (int)fminT((T)(z0 + 1), (T)(unsigned)(d.nz - 1));
    return xw0 * yw0 * zw0 * f[x0 + y0 * sx + z0 * sxy] + xw1 * yw0 * zw0 * f[x1 + y0 * sx + z0 * sxy] +
           xw0 * yw1 * zw0 * f[x0 + y1 * sx + z0 * sxy] + xw1 * yw1 * zw0 * f[x1 + y1 * sx + z0 * sxy] +
           xw0 * yw0 * zw1 * f[x0 + y0 * sx + z1 * sxy] + xw1 * yw0 * zw1 * f[x1 + y0 * sx + z1 * sxy] +
           xw0 * yw1 * zw1 * f[x0 + y1 * sx + z1 * sxy] + xw1 * yw1 * zw1 * f[x1 + y1 * sx + z1 * sxy];
}

// velocityAdvectionU/V/W (:527-615): [now] -> [past], faces with both cells fluid.
template <typename T>
void advect_velocity(const Dims& d, const T* u0, const T* v0, const T* w0, T* u1, T* v1, T* w1,
                     const uint8_t* s, float dt) {
    const T tdt = (T)dt;
    const long long sx = d.nx + 1, sxy = (long long)(d.nx + 1) * (d.ny + 1);
    const T h = (T)0.5f;
#pragma omp parallel for schedule(static)
    for (int z = 1; z < d.nz - 1; ++z)
        for (int y = 1; y < d.ny - 1; ++y)
            for (int x = 1; x < d.nx; ++x)
                if (s[d.c(x, y, z)] != 0 && s[d.c(x - 1, y, z)] != 0) {
                    T xt = (T)x, yt = (T)(y + 0.5), zt = (T)(z + 0.5);
                    T uu = u0[d.f(x, y, z)];
                    T vv = avgV(v0, d, x, y, z);
                    T ww = avgW(w0, d, x, y, z);
                    xt = xt - tdt * uu;
                    yt = yt - tdt * vv;
                    zt = zt - tdt * ww;
                    u1[d.f(x, y, z)] = sample(u0, sx, sxy, xt, yt, zt, (T)0, h, h, d);
                }
#pragma omp parallel for schedule(static)
    for (int z = 1; z < d.nz - 1; ++z)
        for (int y = 1; y < d.ny; ++y)
            for (int x = 1; x < d.nx - 1; ++x)
                if (s[d.c(x, y, z)] != 0 && s[d.c(x, y - 1, z)] != 0) {
                    T xt = (T)(x + 0.5), yt = (T)y, zt = (T)(z + 0.5);
                    T uu = avgU(u0, d, x, y, z);
                    T vv = v0[d.f(x, y, z)];
                    T ww = avgW(w0, d, x, y, z);
                    xt = xt - tdt * uu;
                    yt = yt - tdt * vv;
                    zt = zt - tdt * ww;
                    v1[d.f(x, y, z)] = sample(v0, sx, sxy, xt, yt, zt, h, (T)0, h, d);
                }
#pragma omp parallel for schedule(static)
    for (int z = 1; z < d.nz; ++z)
        for (int y = 1; y < d.ny - 1; ++y)
            for (int x = 1; x < d.nx - 1; ++x)
                if (s[d.c(x, y, z)] != 0 && s[d.c(x, y, z - 1)] != 0) {
                    T xt = (T)(x + 0.5), yt = (T)(y + 0.5), zt = (T)z;
                    T uu = avgU(u0, d, x, y, z);
                    T vv = avgV(v0, d, x, y, z);
                    T ww = w0[d.f(x, y, z)];
                    xt = xt - tdt * uu;
                    yt = yt - tdt * vv;
                    zt = zt - tdt * ww;
                    w1[d.f(x, y, z)] = sample(w0, sx, sxy, xt, yt, zt, h, h, (T)0, d);
                }
}

// advectSmoke (:617-638): uses the NEW velocities; the backtrace is evaluated in double.
template <typename T>
void advect_density(const Dims& d, const T* r0, T* r1, const T* u, const T* v, const T* w,
                    const uint8_t* s, float dt) {
    const T tdt = (T)dt;
    const T h = (T)0.5f;
#pragma omp parallel for schedule(static)
    for (int z = 1; z < d.nz - 1; ++z)
        for (int y = 1; y < d.ny - 1; ++y)
            for (int x = 1; x < d.nx - 1; ++x)
                if (s[d.c(x, y, z)] != 0) {
                    T ut = (u[d.f(x, y, z)] + u[d.f(x + 1, y, z)]) / (T)2;
                    T vt = (v[d.f(x, y, z)] + v[d.f(x, y + 1, z)]) / (T)2;
                    T wt = (w[d.f(x, y, z)] + w[d.f(x, y, z + 1)]) / (T)2;
                    T xt, yt, zt;
                    if (sizeof(T) == sizeof(float)) {
                        xt = (T)((double)x + 0.5 - (double)(ut * tdt));
                        yt = (T)((double)y + 0.5 - (double)(vt * tdt));
                        zt = (T)((double)z + 0.5 - (double)(wt * tdt));
                    } else {
                        xt = (T)x + (T)0.5 - ut * tdt;
                        yt = (T)y + (T)0.5 - vt * tdt;
                        zt = (T)z + (T)0.5 - wt * tdt;
                    }
                    r1[d.c(x, y, z)] =
                        sample(r0, (long long)d.nx, (long long)d.nx * d.ny, xt, yt, zt, h, h, h, d);
                }
}

template <typename T>
float max_div(const Dims& d, const T* u, const T* v, const T* w, const uint8_t* s) {
    T m = 0;
    for (int z = 1; z < d.nz - 1; ++z)
        for (int y = 1; y < d.ny - 1; ++y)
            for (int x = 1; x < d.nx - 1; ++x) {
                if (!projectable(d, s, x, y, z)) continue;
                long long i = d.f(x, y, z);
                T div = -u[i] + u[d.f(x + 1, y, z)] + -v[i] + v[d.f(x, y + 1, z)] + -w[i] +
                        w[d.f(x, y, z + 1)];
                max_abs_bits(div, m);
            }
    return (float)m;
}

// Moving-obstacle boundary (no counterpart in the reference, which stores the obstacles'
// velocity without using it, :299-301): after forcing, every face with a cell of obstacle `o`
// (interior, inside its sphere by fillObstacle's test) on either side takes o's velocity.
template <typename T>
void obstacle_velocity(const Dims& d, T* u, T* v, T* w, const float* o) {
    auto cell = [&](int x, int y, int z) {
        if (x < 1 || y < 1 || z < 1 || x > d.nx - 2 || y > d.ny - 2 || z > d.nz - 2) return false;
        const float dx = (float)x - o[0], dy = (float)y - o[1], dz = (float)z - o[2];
        const float dist = dx * dx + dy * dy + dz * dz;
        return dist < o[6] * o[6];
    };
    for (int z = 0; z <= d.nz; ++z)
        for (int y = 0; y <= d.ny; ++y)
            for (int x = 0; x <= d.nx; ++x) {
                const long long i = d.f(x, y, z);
                const bool c = cell(x, y, z);
                if (x >= 1 && x <= d.nx - 1 && y < d.ny && z < d.nz && (c || cell(x - 1, y, z))) u[i] = (T)o[3];
                if (y >= 1 && y <= d.ny - 1 && x < d.nx && z < d.nz && (c || cell(x, y - 1, z))) v[i] = (T)o[4];
                if (z >= 1 && z <= d.nz - 1 && x < d.nx && y < d.ny && (c || cell(x, y, z - 1))) w[i] = (T)o[5];
            }
}

// FP64-checked refinement after the pressure projection (no counterpart in the reference).  A
// round measures d = ((((-u0 + u1) + -v0) + v1) + -w0) + w1 per projectable cell in double from
// the FP32 faces; when some |d| > tol it solves A e = (float)(-d) from e = 0 with `sweeps`
// red-black sweeps (project_pressure's update), subtracts grad e on fluid-fluid faces and adds e
// to P.  The last round only measures.  T = float only (the FP32 solve it refines).
double measure_div64(const Dims& d, const float* u, const float* v, const float* w, const uint8_t* s,
                     float* b, float* e, bool write, double tol, bool* need) {
    double m = 0.0;
    *need = false;
    for (int z = 0; z < d.nz; ++z)
        for (int y = 0; y < d.ny; ++y)
            for (int x = 0; x < d.nx; ++x) {
                long long c = d.c(x, y, z);
                if (projectable(d, s, x, y, z)) {
                    long long i = d.f(x, y, z);
                    const double dv = ((((-(double)u[i] + (double)u[d.f(x + 1, y, z)]) + -(double)v[i]) +
                                        (double)v[d.f(x, y + 1, z)]) + -(double)w[i]) + (double)w[d.f(x, y, z + 1)];
                    const double a = std::fabs(dv);
                    if (a > m || a != a) m = a;
                    if (a > tol) *need = true;
                    if (write) b[c] = (float)(-dv);
                } else if (write) {
                    b[c] = 0.0f;
                }
                if (write) e[c] = 0.0f;
            }
    return m;
}

void refine_pressure(const Dims& d, float* u, float* v, float* w, float* P, const uint8_t* s, int rounds,
                     int sweeps, double omega, float tol, orc_stats* st) {
    std::vector<float> b((size_t)d.nx * d.ny * d.nz), e((size_t)d.nx * d.ny * d.nz);
    float wacc[7];
    wacc[0] = 0.0f;
    for (int a = 1; a <= 6; ++a) wacc[a] = (float)omega / (float)a;
    bool need = false;
    double m = measure_div64(d, u, v, w, s, b.data(), e.data(), true, (double)tol, &need);
    int applied = 0;
    for (int r = 0; r < rounds && need; ++r) {
        for (int k = 0; k < sweeps; ++k)
            for (int colour = 0; colour < 2; ++colour)
                for (int z = 1; z < d.nz - 1; ++z)
                    for (int y = 1; y < d.ny - 1; ++y)
                        for (int x = 1 + ((1 + y + z + colour) & 1); x < d.nx - 1; x += 2) {
                            if (!projectable(d, s, x, y, z)) continue;
                            const int acc = fluid_nbrs(d, s, x, y, z);
                            const long long c = d.c(x, y, z);
                            const float sum = nbr_sum(d, e.data(), x, y, z);
                            const float rr = fma_t<float>(-(float)acc, e[c], b[c] + sum);
                            e[c] = fma_t<float>(wacc[acc], rr, e[c]);
                        }
        for (int z = 1; z < d.nz - 1; ++z)
            for (int y = 1; y < d.ny - 1; ++y)
                for (int x = 1; x < d.nx; ++x)
                    if (s[d.c(x - 1, y, z)] && s[d.c(x, y, z)]) {
                        long long i = d.f(x, y, z);
                        u[i] = u[i] - (e[d.c(x, y, z)] - e[d.c(x - 1, y, z)]);
                    }
        for (int z = 1; z < d.nz - 1; ++z)
            for (int y = 1; y < d.ny; ++y)
                for (int x = 1; x < d.nx - 1; ++x)
                    if (s[d.c(x, y - 1, z)] && s[d.c(x, y, z)]) {
                        long long i = d.f(x, y, z);
                        v[i] = v[i] - (e[d.c(x, y, z)] - e[d.c(x, y - 1, z)]);
                    }
        for (int z = 1; z < d.nz; ++z)
            for (int y = 1; y < d.ny - 1; ++y)
                for (int x = 1; x < d.nx - 1; ++x)
                    if (s[d.c(x, y, z - 1)] && s[d.c(x, y, z)]) {
                        long long i = d.f(x, y, z);
                        w[i] = w[i] - (e[d.c(x, y, z)] - e[d.c(x, y, z - 1)]);
                    }
        for (size_t c = 0; c < e.size(); ++c) P[c] = P[c] + e[c];
        ++applied;
        m = measure_div64(d, u, v, w, s, b.data(), e.data(), r + 1 < rounds, (double)tol, &need);
    }
    st->refine_rounds = applied;
    st->div64_max = (float)m;
}

// simulate (:774-819): flip, objects, forcing, projection, advection; result in rho[past].
template <typename T>
int step(orc_state* S, const orc_params* p, float dt, orc_stats* st) {
    Dims d{S->nx, S->ny, S->nz};
    int past = S->index_now;
    int now = S->index_now ^ 1;
    S->index_now = now;
    T* rho[2] = {(T*)S->rho[0], (T*)S->rho[1]};
    T* u[2] = {(T*)S->u[0], (T*)S->u[1]};
    T* v[2] = {(T*)S->v[0], (T*)S->v[1]};
    T* w[2] = {(T*)S->w[0], (T*)S->w[1]};
    if (p->n_boxes) emit_boxes<T>(d, rho[0], rho[1], v[now], p->boxes, p->n_boxes);
    fill_smoke<T>(d, rho[0], rho[1], p->spheres, p->n_spheres);
    if (p->n_obstacles) fill_obstacles(d, S->s, p->obstacles, p->n_obstacles);
    forcing<T>(d, u[now], v[now], w[now], rho[now], S->s, dt, p->gravity, p->buoyancy,
               p->clamp_const, p->clamp_mode);
    if (p->obstacle_velocity && p->n_obstacles)
        obstacle_velocity<T>(d, u[now], v[now], w[now], p->obstacles + 7 * (p->n_obstacles - 1));
    orc_stats local{};
    if (p->scheme == 0) {
        project_velocity<T>(d, u[now], v[now], w[now], S->s, p->iterations, p->omega);
        local.sweeps = p->iterations;
    } else {
        project_pressure<T>(d, u[now], v[now], w[now], (T*)S->P, (T*)S->b, S->s, p->iterations,
                            p->omega, p->tol, p->check_every, p->warm_start, &local, p->solver);
        local.div64_max = -1.0f;
        if (p->refine > 0 && p->tol > 0.0f && sizeof(T) == sizeof(float))
            refine_pressure(d, (float*)u[now], (float*)v[now], (float*)w[now], (float*)S->P, S->s, p->refine,
                            p->refine_sweeps, p->omega, p->tol, &local);
    }
    local.div_max = max_div<T>(d, u[now], v[now], w[now], S->s);
    advect_velocity<T>(d, u[now], v[now], w[now], u[past], v[past], w[past], S->s, dt);
    advect_density<T>(d, rho[now], rho[past], u[past], v[past], w[past], S->s, dt);
    if (st) *st = local;
    return 0;
}

}  // namespace

extern "C" {

// Full step on the state (scheme and options in p).  Returns 0.
int orc_f32_step(orc_state* S, const orc_params* p, float dt, orc_stats* st) { return step<float>(S, p, dt, st); }
int orc_f64_step(orc_state* S, const orc_params* p, float dt, orc_stats* st) { return step<double>(S, p, dt, st); }

// Stage entry points (for stage-level parity tests).
void orc_f32_fill_smoke(float* r0, float* r1, int nx, int ny, int nz, const float* sp, int ns) {
    fill_smoke<float>(Dims{nx, ny, nz}, r0, r1, sp, ns);
}
void orc_f32_emit_boxes(float* r0, float* r1, float* v_now, int nx, int ny, int nz, const float* bx, int nb) {
    emit_boxes<float>(Dims{nx, ny, nz}, r0, r1, v_now, bx, nb);
}
void orc_fill_obstacles(uint8_t* s, int nx, int ny, int nz, const float* ob, int no) {
    fill_obstacles(Dims{nx, ny, nz}, s, ob, no);
}
void orc_f32_forcing(float* u, float* v, float* w, const float* rho, const uint8_t* s, int nx, int ny,
                     int nz, float dt, float g, float a, float clamp_const, int clamp_mode) {
    forcing<float>(Dims{nx, ny, nz}, u, v, w, rho, s, dt, g, a, clamp_const, clamp_mode);
}
void orc_f32_project_velocity(float* u, float* v, float* w, const uint8_t* s, int nx, int ny, int nz,
                              int iters, double omega) {
    project_velocity<float>(Dims{nx, ny, nz}, u, v, w, s, iters, omega);
}
int orc_f32_project_pressure(float* u, float* v, float* w, float* P, float* b, const uint8_t* s, int nx,
                             int ny, int nz, int max_sweeps, double omega, float tol, int check_every,
                             int warm_start, orc_stats* st) {
    return project_pressure<float>(Dims{nx, ny, nz}, u, v, w, P, b, s, max_sweeps, omega, tol,
                                   check_every, warm_start, st);
}
int orc_f64_project_pressure(double* u, double* v, double* w, double* P, double* b, const uint8_t* s,
                             int nx, int ny, int nz, int max_sweeps, double omega, float tol,
                             int check_every, int warm_start, orc_stats* st) {
    return project_pressure<double>(Dims{nx, ny, nz}, u, v, w, P, b, s, max_sweeps, omega, tol,
                                    check_every, warm_start, st);
}
void orc_f32_advect_velocity(const float* u0, const float* v0, const float* w0, float* u1, float* v1,
                             float* w1, const uint8_t* s, int nx, int ny, int nz, float dt) {
    advect_velocity<float>(Dims{nx, ny, nz}, u0, v0, w0, u1, v1, w1, s, dt);
}
void orc_f32_advect_density(const float* r0, float* r1, const float* u, const float* v, const float* w,
                            const uint8_t* s, int nx, int ny, int nz, float dt) {
    advect_density<float>(Dims{nx, ny, nz}, r0, r1, u, v, w, s, dt);
}
float orc_f32_max_div(const float* u, const float* v, const float* w, const uint8_t* s, int nx, int ny, int nz) {
    return max_div<float>(Dims{nx, ny, nz}, u, v, w, s);
}
float orc_f64_max_div(const double* u, const double* v, const double* w, const uint8_t* s, int nx, int ny,
                      int nz) {
    return max_div<double>(Dims{nx, ny, nz}, u, v, w, s);
}

}  // extern "C"
