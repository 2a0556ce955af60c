// Device-side building blocks of the GB300 SPH particle loop: smoothing
// kernels, the cell-grid neighbour walk and deterministic block reductions.
//
// Two numeric forms share this code (template parameter R):
//   R = double  parity form: absolute positions, the reference's expression
//               order and IEEE division, for checks against the CPU solver;
//   R = float   production form: positions stored relative to the corner of
//               the particle's grid cell (cell index kept as an integer), so
//               pair distances keep ~ulp(h) precision anywhere in the domain.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace sph {

// ---------------------------------------------------------------------------
// Vector types
// ---------------------------------------------------------------------------
template <typename R> struct alignas(4 * sizeof(R)) P4 { R x, y, z, w; };
template <typename R> struct V3 { R x, y, z; };

template <typename R> __host__ __device__ __forceinline__ V3<R> v3(R x, R y, R z) { return V3<R>{x, y, z}; }
template <typename R> __device__ __forceinline__ V3<R> operator+(V3<R> a, V3<R> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <typename R> __device__ __forceinline__ V3<R> operator-(V3<R> a, V3<R> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <typename R> __device__ __forceinline__ V3<R> operator*(R s, V3<R> a) { return {s * a.x, s * a.y, s * a.z}; }
template <typename R> __device__ __forceinline__ V3<R> operator*(V3<R> a, R s) { return {a.x * s, a.y * s, a.z * s}; }
template <typename R> __device__ __forceinline__ V3<R> operator/(V3<R> a, R s) { return {a.x / s, a.y / s, a.z / s}; }
template <typename R> __device__ __forceinline__ V3<R> operator-(V3<R> a) { return {-a.x, -a.y, -a.z}; }
// (x*x' + y*y') + z*z', the order GLM's dot uses
template <typename R> __device__ __forceinline__ R dot3(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <typename R> __device__ __forceinline__ V3<R> xyz(const P4<R>& p) { return {p.x, p.y, p.z}; }

__device__ __forceinline__ P4<float> ldg4(const P4<float>* p)
{
    float4 t = __ldg(reinterpret_cast<const float4*>(p));
    return P4<float>{t.x, t.y, t.z, t.w};
}
__device__ __forceinline__ P4<double> ldg4(const P4<double>* p)
{
    const double2* q = reinterpret_cast<const double2*>(p);
    double2 a = __ldg(q), b = __ldg(q + 1);
    return P4<double>{a.x, a.y, b.x, b.y};
}
template <typename R> __device__ __forceinline__ R ldg1(const R* p) { return __ldg(p); }
// Streaming load (evict first): data read exactly once, such as pair-list
// records, so that it does not displace the neighbour data that the gathers
// of the same pass re-use from L1.
__device__ __forceinline__ P4<float> ldcs4(const P4<float>* p)
{
    // read-only and not allocated in L1, which keeps the gathered neighbour
    // fields
    float4 t;
    asm("ld.global.nc.L1::no_allocate.v4.f32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(t.x), "=f"(t.y), "=f"(t.z), "=f"(t.w)
                 : "l"(p));
    return P4<float>{t.x, t.y, t.z, t.w};
}
__device__ __forceinline__ P4<double> ldcs4(const P4<double>* p)
{
    const double2* q = reinterpret_cast<const double2*>(p);
    double2 a = __ldcs(q), b = __ldcs(q + 1);
    return P4<double>{a.x, a.y, b.x, b.y};
}

// Division by the support radius: IEEE division in the parity form (the
// reference divides), multiplication by 1/h in the production form.
__device__ __forceinline__ double div_h(double r, double h, double) { return r / h; }
__device__ __forceinline__ float div_h(float r, float, float inv_h) { return r * inv_h; }

// ---------------------------------------------------------------------------
// Per-scene constants (kernel coefficients as each reference kernel's
// setSupportRadius computes them, evaluated in double on the host).
// ---------------------------------------------------------------------------
template <typename R> struct Consts {
    R h, inv_h, h2, cull2;
    R cs_k, cs_l;                  // CubicSpline.h:18-26
    R p6_h2, p6_value, p6_grad;    // Poly6.h:19-28
    R sp_value, sp_grad;           // Spiky.h:18-27
    R vk_lapl;                     // ViscoK.h:18-26
    R co_c1, co_c2;                // Cohesion.h:20-27
    R mass, density0, eps;
    R gx, gy, gz;
    R stiffness, gamma, k_eos;     // k_eos = stiffness * density0 / gamma
    R visc, bvisc, st, adh;
    R cube_min[3], cube_max[3];
    R bwarm;                       // warm-start boundary factor: 2 (Akinci), 1 (PCISPH model)
    R bh_nf, bh_tf;                // PCISPH boundary model normal / tangential factors
    double inv_density0;           // 1 / density0 (FP32 form's error reductions)
    int force_flags;
    int has_cube;
};

// A particle's relative error x / density0 for the solver loops' average:
// the reference's FP64 division in the parity form, a multiplication by the
// reciprocal in the FP32 form (FP64 division is slow on this part).
template <typename R> __device__ __forceinline__ double rel_error(const Consts<R>& c, double x)
{
    if constexpr (sizeof(R) == 8) return x / (double)c.density0;
    else return x * c.inv_density0;
}

enum ForceFlags : int {
    F_XSPH = 1, F_STD_VISC = 2, F_ART_VISC = 4, F_SURFACE_TENSION = 8, F_ADHESION = 16, F_BVISC = 32,
};

// Scalars that change during a run and live on the device so that whole
// steps run without host round trips (the CFL step writes dt, reductions
// write the errors and the loop flags).
struct DevScalars {
    double dt, time;
    double avgDensError, avgDivError, maxDensityError;
    double maxVel;
    double scaling;                // PCISPH delta
    unsigned iterations, iterationsV, next_active;
    unsigned active;               // loop flag of the solve in progress
    unsigned steps;
    unsigned long long sumIterations, sumIterationsV;
    unsigned status;               // SPH_STATUS_* bits
    unsigned block_counter;        // last-block-done counter of reductions
    unsigned grid_epoch;           // grid builds so far (cell lifetimes, PCISPH boundary model)
    unsigned n_active;             // active fluid particles (grows when emitters emit)
    unsigned escaped;              // a particle was kept in a border cell since the last grid growth
    unsigned disp_bits;            // PCISPH: largest predicted displacement of the loop so far (float bits)
};

enum StatusBits : unsigned {
    ST_OUT_OF_GRID = 1u, ST_NONFINITE = 2u, ST_ITER_CAP = 4u, ST_ITER_CAP_V = 8u, ST_DIVERGED = 16u,
    ST_BOUNDS = 32u,
};

// Index checks of the bounds-checked build (compiled with -DSPH_BOUNDS_CHECK,
// libsph_gb300_checked.so): a neighbour index read from device data (a pair
// record, a candidate list entry) that is not below its array's length sets
// ST_BOUNDS in *FAULT and the access is skipped.  In the ordinary build the
// check is the constant true and compiles away.
#ifdef SPH_BOUNDS_CHECK
#define SPH_INDEX_OK(j, n, fault) ((j) < (n) ? true : ((fault) ? (atomicOr((fault), ST_BOUNDS), false) : false))
#else
#define SPH_INDEX_OK(j, n, fault) true
#endif

// Solver limits used by the device-side loop controls.
struct LoopLimits {
    double maxError, maxErrorV;
    unsigned minIt, maxIt, minItV, maxItV;
    double cflFactor, particleRadius, minTs, maxTs;
};

// ---------------------------------------------------------------------------
// Grid: dense cell box around the domain.  A cell (cx, cy, cz) sits in
// column col = morton(cx, cy); cells of a column are consecutive in z, so the
// three cells z-1..z+1 of a neighbour column are one contiguous particle
// range, visited in the reference's x -> y -> z offset order
// (HashTable.h:147-167).  key = col * nz + cz.
// ---------------------------------------------------------------------------
struct GridView {
    int nx, ny, nz;
    int ox, oy, oz;                 // absolute cell index of grid cell (0,0,0)
    const uint32_t* mortx;          // spread bits of cx
    const uint32_t* morty;          // spread bits of cy
};

__device__ __forceinline__ uint32_t pack_cell(int cx, int cy, int cz) { return (uint32_t)cx | ((uint32_t)cy << 11) | ((uint32_t)cz << 22); }
__device__ __forceinline__ int cell_x(uint32_t c) { return (int)(c & 2047u); }
__device__ __forceinline__ int cell_y(uint32_t c) { return (int)((c >> 11) & 2047u); }
__device__ __forceinline__ int cell_z(uint32_t c) { return (int)(c >> 22); }
__device__ __forceinline__ uint32_t cell_key(const GridView& g, int cx, int cy, int cz)
{
    return (__ldg(g.mortx + cx) | __ldg(g.morty + cy)) * (uint32_t)g.nz + (uint32_t)cz;
}

// Visit every candidate j of the 27 cells around the particle's cell, calling
// f(j, s) with s the particle's position expressed in the frame of j's cell
// (so that r_ij = s - pos_j), in the reference's x -> y -> z cell order.
//
// One lane per particle (G == 1): the cell starts of all nine neighbour
// columns are fetched first (independent loads, one latency instead of nine
// chained ones), then each column's contiguous particle range is streamed;
// in the cell-relative form the frame of candidate j (its z cell within the
// column) is picked by comparing j with the column's two inner cell starts.
// Columns and z-cells whose box lies farther than h from the particle are
// skipped: they hold no neighbour, and every smoothing kernel is zero there,
// so the sums are those of the full 27-cell walk.  TRIM = false walks all 27
// cells: needed where the distance is taken to positions other than the ones
// the candidates are filed by (PCISPH's predicted positions, filed by their
// current cells).
// G > 1 lanes split each cell's range (lane l takes every G-th candidate).
// ROLLED (G = 1): the nine columns one after another, each column's range
// looked up just before it is walked, the visit code emitted once (the
// same candidates in the same order; smaller code, fewer live registers).
template <typename R, int G, bool TRIM = true, bool ROLLED = false, typename F>
__device__ __forceinline__ void walk(const GridView& g, const uint32_t* __restrict__ starts, uint32_t pc, V3<R> xi, R h,
                                     int lane, F&& f)
{
    constexpr bool REL = sizeof(R) == 4;
    const int cx = cell_x(pc), cy = cell_y(pc), cz = cell_z(pc);
    const int z0 = cz > 0 ? cz - 1 : 0;
    const int z1 = cz + 1 < g.nz ? cz + 1 : g.nz - 1;
    if constexpr (G == 1 && ROLLED) {
        const R ofx = REL ? xi.x : xi.x - (R)(cx + g.ox) * h;
        const R ofy = REL ? xi.y : xi.y - (R)(cy + g.oy) * h;
        const R ofz = REL ? xi.z : xi.z - (R)(cz + g.oz) * h;
        const R gxm = ofx > (R)0 ? ofx * ofx : (R)0, gxp = h - ofx > (R)0 ? (h - ofx) * (h - ofx) : (R)0;
        const R gym = ofy > (R)0 ? ofy * ofy : (R)0, gyp = h - ofy > (R)0 ? (h - ofy) * (h - ofy) : (R)0;
        const R gzm = ofz > (R)0 ? ofz * ofz : (R)0, gzp = h - ofz > (R)0 ? (h - ofz) * (h - ofz) : (R)0;
        const R lim = TRIM ? h * h * (R)(1.0 + 1e-5) : (R)INFINITY;
        const R szm = xi.z + h, sz0 = xi.z, szp = xi.z - h;
#pragma unroll 1
        for (int c = 0; c < 9; ++c) {
            const int dx = c / 3 - 1, dy = c - (c / 3) * 3 - 1;
            const int x = cx + dx, y = cy + dy;
            const R gxy = (dx < 0 ? gxm : (dx > 0 ? gxp : (R)0)) + (dy < 0 ? gym : (dy > 0 ? gyp : (R)0));
            if (x < 0 || x >= g.nx || y < 0 || y >= g.ny || !(gxy <= lim)) continue;
            const uint32_t base = (__ldg(g.mortx + x) | __ldg(g.morty + y)) * (uint32_t)g.nz;
            const uint32_t s0 = __ldg(starts + base + z0), sm = __ldg(starts + base + cz);
            const uint32_t sp = __ldg(starts + base + cz + 1), s1 = __ldg(starts + base + z1 + 1);
            const uint32_t bb = gxy + gzm <= lim ? s0 : sm;
            const uint32_t ee = gxy + gzp <= lim ? s1 : sp;
            V3<R> s = REL ? V3<R>{xi.x - (R)dx * h, xi.y - (R)dy * h, xi.z} : xi;
#pragma unroll 1
            for (uint32_t j = bb; j < ee; ++j) {
                if (REL) s.z = j < sm ? szm : (j < sp ? sz0 : szp);
                f(j, s);
            }
        }
    } else if constexpr (G == 1) {
        // the particle's offset inside its own cell, and the squared gap from
        // it to each neighbour layer (0 for its own layer): a cell whose box
        // is farther than h from the particle holds no neighbour
        const R ofx = REL ? xi.x : xi.x - (R)(cx + g.ox) * h;
        const R ofy = REL ? xi.y : xi.y - (R)(cy + g.oy) * h;
        const R ofz = REL ? xi.z : xi.z - (R)(cz + g.oz) * h;
        const R gxm = ofx > (R)0 ? ofx * ofx : (R)0, gxp = h - ofx > (R)0 ? (h - ofx) * (h - ofx) : (R)0;
        const R gym = ofy > (R)0 ? ofy * ofy : (R)0, gyp = h - ofy > (R)0 ? (h - ofy) * (h - ofy) : (R)0;
        const R gzm = ofz > (R)0 ? ofz * ofz : (R)0, gzp = h - ofz > (R)0 ? (h - ofz) * (h - ofz) : (R)0;
        const R lim = TRIM ? h * h * (R)(1.0 + 1e-5) : (R)INFINITY;
        uint32_t b[9], m0[9], m1[9], e[9];
#pragma unroll
        for (int dx = -1; dx <= 1; ++dx) {
            const int x = cx + dx;
            const bool okx = x >= 0 && x < g.nx;
            const uint32_t mx = okx ? __ldg(g.mortx + x) : 0u;
            const R gx = dx < 0 ? gxm : (dx > 0 ? gxp : (R)0);
#pragma unroll
            for (int dy = -1; dy <= 1; ++dy) {
                const int c = (dx + 1) * 3 + (dy + 1);
                const int y = cy + dy;
                const R gxy = gx + (dy < 0 ? gym : (dy > 0 ? gyp : (R)0));
                const bool ok = okx && y >= 0 && y < g.ny && gxy <= lim;
                const uint32_t base = ok ? (mx | __ldg(g.morty + y)) * (uint32_t)g.nz : 0u;
                if (ok) {
                    const uint32_t s0 = __ldg(starts + base + z0), sm = __ldg(starts + base + cz);
                    const uint32_t sp = __ldg(starts + base + cz + 1), s1 = __ldg(starts + base + z1 + 1);
                    b[c] = gxy + gzm <= lim ? s0 : sm;   // cell cz-1 only if within reach
                    e[c] = gxy + gzp <= lim ? s1 : sp;   // cell cz+1 only if within reach
                    m0[c] = sm;
                    m1[c] = sp;
                } else {
                    b[c] = 0u; e[c] = 0u; m0[c] = 0u; m1[c] = 0u;
                }
            }
        }
        const R szm = xi.z + h, sz0 = xi.z, szp = xi.z - h;  // frames of cells cz-1, cz, cz+1
#pragma unroll
        for (int c = 0; c < 9; ++c) {
            const int dx = c / 3 - 1, dy = c % 3 - 1;
            // absolute form: every candidate is compared with xi itself
            V3<R> s = REL ? V3<R>{xi.x - (R)dx * h, xi.y - (R)dy * h, xi.z} : xi;
            const uint32_t bb = b[c], ee = e[c];
#pragma unroll 1
            for (uint32_t j = bb; j < ee; ++j) {
                if (REL) s.z = j < m0[c] ? szm : (j < m1[c] ? sz0 : szp);
                f(j, s);
            }
        }
    } else {
#pragma unroll
        for (int dx = -1; dx <= 1; ++dx) {
            const int x = cx + dx;
            if (x < 0 || x >= g.nx) continue;
            const uint32_t mx = __ldg(g.mortx + x);
#pragma unroll
            for (int dy = -1; dy <= 1; ++dy) {
                const int y = cy + dy;
                if (y < 0 || y >= g.ny) continue;
                const uint32_t base = (mx | __ldg(g.morty + y)) * (uint32_t)g.nz;
                if constexpr (REL) {
                    const R sx = xi.x - (R)dx * h, sy = xi.y - (R)dy * h;
                    uint32_t bz = __ldg(starts + base + z0);
                    for (int z = z0; z <= z1; ++z) {
                        const uint32_t ez = __ldg(starts + base + z + 1);
                        const V3<R> s = {sx, sy, xi.z - (R)(z - cz) * h};
                        for (uint32_t j = bz + lane; j < ez; j += G) f(j, s);
                        bz = ez;
                    }
                } else {
                    const uint32_t bz = __ldg(starts + base + z0), ez = __ldg(starts + base + z1 + 1);
                    for (uint32_t j = bz + lane; j < ez; j += G) f(j, xi);
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Smoothing kernels
// ---------------------------------------------------------------------------

// W and grad W of one pair from the squared distance, for the pair-list
// build.  FAST (FP32 form): 1/|r| from the hardware reciprocal square root
// (a few ulp) replaces the correctly rounded sqrt and division; the
// polynomials are those of cubic_W / cubic_gradW.
template <bool FAST, typename R>
__device__ __forceinline__ void cubic_W_gradW(const Consts<R>& c, V3<R> r, R r2, R* w, V3<R>* grad)
{
    if constexpr (FAST && sizeof(R) == 4) {
        const float rinv = rsqrtf(r2);
        const float rl = r2 > 0.f ? r2 * rinv : 0.f;
        const float q = rl * c.inv_h;
        float res = 0.f;
        V3<float> g = {0.f, 0.f, 0.f};
        if (q <= 1.f) {
            const V3<float> gradq = r * (rinv * c.inv_h);
            if (q <= 0.5f) {
                const float q2 = q * q;
                res = c.cs_k * (6.f * (q2 * q) - 6.f * q2 + 1.f);
                g = (c.cs_l * q * (3.f * q - 2.f)) * gradq;
            } else {
                const float fq = 1.f - q;
                res = c.cs_k * (2.f * (fq * fq * fq));
                g = (c.cs_l * (-fq * fq)) * gradq;
            }
            if (!(rl > 1.0e-5f)) g = V3<float>{0.f, 0.f, 0.f};
        }
        *w = res;
        *grad = g;
    } else {
        *w = cubic_W(c, sqrt(r2));
        *grad = cubic_gradW(c, r, r2);
    }
}

// Poly6::W Poly6.h:30-43 from the squared distance (the length is formed and
// squared again, as the reference does).
template <typename R> __device__ __forceinline__ R poly6_W(const Consts<R>& c, R r2)
{
    const R mod_r = sqrt(r2);
    const R mod_r2 = mod_r * mod_r;
    if (mod_r2 <= c.p6_h2) {
        const R diff = c.p6_h2 - mod_r2;
        return c.p6_value * diff * diff * diff;
    }
    return (R)0;
}

// CubicSpline::W CubicSpline.h:28-46, from the distance r.
template <typename R> __device__ __forceinline__ R cubic_W(const Consts<R>& c, R r)
{
    R res = 0;
    const R q = div_h(r, c.h, c.inv_h);
    if (q <= (R)1) {
        if (q <= (R)0.5) {
            const R q2 = q * q;
            const R q3 = q2 * q;
            res = c.cs_k * ((R)6 * q3 - (R)6 * q2 + (R)1);
        } else {
            const R f = (R)1 - q;
            res = c.cs_k * ((R)2 * (f * f * f));
        }
    }
    return res;
}

// CubicSpline::gradW CubicSpline.h:53-73, given r and |r|^2.
template <typename R> __device__ __forceinline__ V3<R> cubic_gradW(const Consts<R>& c, V3<R> r, R r2)
{
    V3<R> res = {0, 0, 0};
    const R rl = sqrt(r2);
    const R q = div_h(rl, c.h, c.inv_h);
    if ((rl > (R)1.0e-5) && (q <= (R)1)) {
        const V3<R> gradq = r * ((R)1 / (rl * c.h));
        if (q <= (R)0.5) {
            res = (c.cs_l * q * ((R)3 * q - (R)2)) * gradq;
        } else {
            const R factor = (R)1 - q;
            res = (c.cs_l * (-factor * factor)) * gradq;
        }
    }
    return res;
}

// Spiky::gradW Spiky.h:43-55
template <typename R> __device__ __forceinline__ V3<R> spiky_gradW(const Consts<R>& c, V3<R> r, R r2)
{
    const R mod_r = sqrt(r2);
    if (mod_r != (R)0 && mod_r <= c.h) {
        const R diff = c.h - mod_r;
        return (-c.sp_grad * diff * diff / mod_r) * r;
    }
    return V3<R>{0, 0, 0};
}

// ViscoK::laplW ViscoK.h:27-35
template <typename R> __device__ __forceinline__ R visc_laplW(const Consts<R>& c, R r2)
{
    const R mod_r = sqrt(r2);
    if (mod_r <= c.h) return c.vk_lapl * (c.h - mod_r);
    return 0;
}

// Cohesion::W Cohesion.h:29-40
template <typename R> __device__ __forceinline__ R cohesion_W(const Consts<R>& c, R mod_r)
{
    R value = 0;
    const R sr = c.h;
    if (((R)2 * mod_r > sr) && (mod_r <= sr)) {
        const R a = sr - mod_r;
        value = c.co_c1 * (a * a * a) * (mod_r * mod_r * mod_r);
    } else if ((mod_r > (R)0) && ((R)2 * mod_r <= sr)) {
        const R a = sr - mod_r;
        value = c.co_c1 * (R)2 * (a * a * a) * (mod_r * mod_r * mod_r) - c.co_c2;
    }
    return value;
}

// Adhesion::W Adhesion.h:23-35 (the reference never applies its valueCoef)
template <typename R> __device__ __forceinline__ R adhesion_W(const Consts<R>& c, R mod_r)
{
    const R sr = c.h;
    if (((R)2 * mod_r > sr) && (mod_r <= sr)) {
        const R value = (R)-4 * mod_r * mod_r / sr + (R)6 * mod_r - (R)2 * sr;
        return sqrt(sqrt(value));   // value^(1/4)
    }
    return 0;
}

// ---------------------------------------------------------------------------
// Block reductions in FP64 with a deterministic last-block finish.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_max(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}

// Sum (or max) of v over the block; the result is valid in thread 0.
template <bool MAX> __device__ __forceinline__ double block_reduce(double v, double* sh)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    v = MAX ? warp_max(v) : warp_sum(v);
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    if (wid == 0) {
        double t = lane < nw ? sh[lane] : (MAX ? -1.0e300 : 0.0);
        t = MAX ? warp_max(t) : warp_sum(t);
        if (lane == 0) sh[0] = t;
    }
    __syncthreads();
    const double r = sh[0];
    __syncthreads();
    return r;
}

// Writes this block's partial and returns true in exactly one block (the
// last to finish), in which every thread sees the total in *total_out.  The
// total is summed in block-index order, so the result does not depend on
// which block finished last.
template <bool MAX>
__device__ __forceinline__ bool finish_reduction(double v, double* partials, unsigned* counter, double* sh,
                                                 double* total_out)
{
    const double b = block_reduce<MAX>(v, sh);
    __shared__ bool is_last;
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = b;
        __threadfence();
        const unsigned done = atomicAdd(counter, 1u);
        is_last = (done == gridDim.x - 1);
    }
    __syncthreads();
    if (!is_last) return false;
    __threadfence();
    double t = MAX ? -1.0e300 : 0.0;
    for (unsigned i = threadIdx.x; i < gridDim.x; i += blockDim.x) {
        const double p = *((volatile double*)(partials + i));
        t = MAX ? fmax(t, p) : t + p;
    }
    const double tot = block_reduce<MAX>(t, sh);
    if (threadIdx.x == 0) *counter = 0u;
    *total_out = tot;
    return true;
}

}  // namespace sph
