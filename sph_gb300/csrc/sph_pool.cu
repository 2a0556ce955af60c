// Batched multi-scene pool: many independent DFSPH scenes advanced together.
//
// All resident scenes share one set of device arrays.  Each scene keeps its
// own dense cell box and a disjoint range of grid keys, so one counting sort
// per step sorts every scene at once and leaves each scene's particles
// contiguous (scenes are laid out in key order).  Per-scene constants, time
// step, solver scalars and loop flags live in a device scene table; every
// kernel looks up its particle's scene.  The solver loops run while any
// scene's loop is active; a scene whose loop has converged skips the
// remaining iterations, exactly as if it ran alone.  Per-scene error sums
// are accumulated as 64-bit fixed-point integers (integer addition is
// associative), so a scene's results do not depend on which other scenes
// share the pool or how its particles fall into blocks.
//
// The scene set changes only between steps (continuous batching): pending
// admissions and removals are applied by a re-layout that repacks the
// resident scenes' state, uploads the new scenes, sorts the boundary and
// rebuilds the grids and pair lists; the per-step CUDA graph is then
// re-captured.
//
// Scenes use the DFSPH solver (DFSPHSolver.cpp) with Akinci boundaries and
// optional XSPH / standard / artificial viscosity, in the FP32 form with pair
// lists (sph_lists.cuh).
#include <cuda_runtime.h>

#include <sys/stat.h>

#include <algorithm>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <list>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "sph_scene.cuh"

struct sph_pool;

namespace sph {

constexpr double kFixScale = 268435456.0;  // 2^28: per-particle error quantum 3.7e-9
// A scene's fixed-point error sum holds at most 2^64 / 2^28 = 6.9e10: with
// n particles, a particle error above kErrBudget / n is not added (the sum
// then cannot wrap) and marks the scene as blown up.  For the largest scenes
// served (4M particles) that is an error of 15,000 (a density of 15,000 rest
// densities, or a divergence error of 15,000 / s); for the mix's 64k, 9e5.
constexpr double kErrBudget = 6.0e10;

struct PoolScene {
    Consts<float> c;
    GridView g;
    LoopLimits lim;
    DevScalars s;
    unsigned long long acc;   // fixed-point error sum of the reduction in progress
    uint32_t key_base, n, nb, pbase, bbase;
    uint32_t running;         // steps left > 0
    uint32_t loop_active;     // this scene's solver loop is still iterating
    uint32_t steps_left;
    uint32_t vmax_bits;       // CFL: max of sqrt(|v|) as float bits
    uint32_t bad;             // reduction in progress saw: 1 a NaN / Inf error, 2 an error above eclamp
    float eclamp;             // kErrBudget / n: largest error a particle adds to the fixed-point sum
    int akinci;
};

struct PoolCounters {
    unsigned any;                       // some scene's loop is active
    unsigned faults;                    // ST_BOUNDS of the bounds-checked build (any scene)
    unsigned long long body_d, body_v;  // loop bodies executed (density / divergence)
};

__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Adds v to scene s's accumulator; all lanes of the warp must call it
// (s = ~0u: nothing to add).  Warps whose lanes share one scene add once.
__device__ __forceinline__ void seg_add(uint32_t s, unsigned long long v, PoolScene* T)
{
    const uint32_t s0 = __shfl_sync(0xffffffffu, s, 0);
    if (__all_sync(0xffffffffu, s == s0)) {
        v = warp_sum_u64(v);
        if ((threadIdx.x & 31) == 0 && s0 != ~0u && v) atomicAdd(&T[s0].acc, v);
    } else if (s != ~0u && v) {
        atomicAdd(&T[s].acc, v);
    }
}

__device__ __forceinline__ unsigned long long to_fixed(double e) { return (unsigned long long)(e * kFixScale + 0.5); }

// A particle's relative error (>= 0) as its fixed-point contribution to its
// scene's sum; a NaN / Inf error or one above the scene's clamp is not
// added, and marks the scene's reduction instead (k_pool_control then reads
// the scene's average as NaN or +Inf, as an FP64 sum of the same terms would).
__device__ __forceinline__ unsigned long long error_contribution(float e, PoolScene& sd)
{
    if (e <= sd.eclamp) return to_fixed((double)e);
    atomicOr(&sd.bad, isfinite(e) ? 2u : 1u);
    return 0ull;
}

__device__ __forceinline__ uint32_t find_segment(const uint32_t* __restrict__ base, uint32_t S, uint32_t i)
{
    uint32_t lo = 0, hi = S;  // last segment whose base <= i
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (base[mid] <= i) lo = mid; else hi = mid;
    }
    return lo;
}

// Bounding box of n points (xyz FP64), points with a non-finite coordinate
// left out (the grid planner's rule): per block {lo xyz, hi xyz} at
// part[6 * blockIdx.x], reduced over the blocks by the host.
constexpr int kBoxBlocks = 64;
__global__ void __launch_bounds__(256) k_point_box(const double* __restrict__ p, uint32_t n, double* __restrict__ part)
{
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double x = p[3 * (size_t)i], y = p[3 * (size_t)i + 1], z = p[3 * (size_t)i + 2];
        if (isfinite(x) && isfinite(y) && isfinite(z)) {
            lo[0] = fmin(lo[0], x); lo[1] = fmin(lo[1], y); lo[2] = fmin(lo[2], z);
            hi[0] = fmax(hi[0], x); hi[1] = fmax(hi[1], y); hi[2] = fmax(hi[2], z);
        }
    }
    __shared__ double sh[6][8];
    for (int k = 0; k < 3; ++k) {
        for (int o = 16; o > 0; o >>= 1) {
            lo[k] = fmin(lo[k], __shfl_down_sync(0xffffffffu, lo[k], o));
            hi[k] = fmax(hi[k], __shfl_down_sync(0xffffffffu, hi[k], o));
        }
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0)
        for (int k = 0; k < 3; ++k) { sh[k][w] = lo[k]; sh[3 + k][w] = hi[k]; }
    __syncthreads();
    if (threadIdx.x < 6) {
        const int k = threadIdx.x;
        double v = sh[k][0];
        for (int j = 1; j < (int)(blockDim.x >> 5); ++j) v = k < 3 ? fmin(v, sh[k][j]) : fmax(v, sh[k][j]);
        part[6 * blockIdx.x + k] = v;
    }
}

// Scene id of every particle of a layout: segments [base[s], base[s] + len[s]).
__global__ void k_fill_sid(uint32_t N, const uint32_t* __restrict__ base, uint32_t S, uint32_t* __restrict__ sid)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < N) sid[i] = find_segment(base, S, i);
}

// Copy of the state carried across a re-layout: scene k's segment moves from
// src_base[k] to dst_base[k] (dst bases ascending).
__global__ void k_repack_fluid(uint32_t N, const uint32_t* __restrict__ dst_base, const uint32_t* __restrict__ src_base,
                               const uint32_t* __restrict__ len, uint32_t S, Fluid<float> src, Fluid<float> dst)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N || S == 0) return;
    const uint32_t k = find_segment(dst_base, S, i);
    const uint32_t off = i - dst_base[k];
    if (off >= len[k]) return;
    const uint32_t j = src_base[k] + off;
    dst.pos[i] = src.pos[j];
    dst.vel[i] = src.vel[j];
    dst.kappa[i] = src.kappa[j];
    dst.kappav[i] = src.kappav[j];
    dst.pred[i] = src.pred[j];
    dst.cell[i] = src.cell[j];
    dst.id[i] = src.id[j];
}

__global__ void k_repack_boundary(uint32_t N, const uint32_t* __restrict__ dst_base, const uint32_t* __restrict__ src_base,
                                  const uint32_t* __restrict__ len, uint32_t S, Boundary<float> src, Boundary<float> dst)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N || S == 0) return;
    const uint32_t k = find_segment(dst_base, S, i);
    const uint32_t off = i - dst_base[k];
    if (off >= len[k]) return;
    const uint32_t j = src_base[k] + off;
    dst.pos[i] = src.pos[j];
    dst.cell[i] = src.cell[j];
    dst.id[i] = src.id[j];
}

// Cells and keys (scene key base + column-Morton key) of every particle;
// MOVE first advances positions of running scenes (updatePositions).
template <bool MOVE>
__global__ void k_pool_cell_update(uint32_t N, Fluid<float> f, const uint32_t* __restrict__ sid, PoolScene* T,
                                   uint32_t* __restrict__ key, uint32_t* __restrict__ slot, uint32_t* __restrict__ count)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    PoolScene& sd = T[sid[i]];
    P4<float> p = f.pos[i];
    if (MOVE && sd.running) {
        const float dt = (float)sd.s.dt;
        const P4<float> v = f.vel[i];
        p.x = p.x + v.x * dt; p.y = p.y + v.y * dt; p.z = p.z + v.z * dt;
    }
    // a NaN / Inf position or velocity never meets a neighbour, so no solver
    // sum would notice it: flag it here (the scene is retired at step end)
    if (!(isfinite(p.x) && isfinite(p.y) && isfinite(p.z))) atomicOr(&sd.s.status, (unsigned)ST_NONFINITE);
    const GridView& g = sd.g;
    const float h = sd.c.h;
    const uint32_t c0 = f.cell[i];
    const int x0 = cell_x(c0), y0 = cell_y(c0), z0 = cell_z(c0);
    const int cx = x0 + (int)floorf(p.x / h), cy = y0 + (int)floorf(p.y / h), cz = z0 + (int)floorf(p.z / h);
    const int ccx = min(max(cx, 0), g.nx - 1), ccy = min(max(cy, 0), g.ny - 1), ccz = min(max(cz, 0), g.nz - 1);
    if (ccx != cx || ccy != cy || ccz != cz) atomicOr(&sd.s.status, (unsigned)ST_OUT_OF_GRID);
    p.x -= (float)(ccx - x0) * h; p.y -= (float)(ccy - y0) * h; p.z -= (float)(ccz - z0) * h;
    if (ccx == cx) p.x = fminf(fmaxf(p.x, 0.f), __int_as_float(__float_as_int(h) - 1));
    if (ccy == cy) p.y = fminf(fmaxf(p.y, 0.f), __int_as_float(__float_as_int(h) - 1));
    if (ccz == cz) p.z = fminf(fmaxf(p.z, 0.f), __int_as_float(__float_as_int(h) - 1));
    p.w = zframe3(p.z, ccz, h);
    f.pos[i] = p;
    f.cell[i] = pack_cell(ccx, ccy, ccz);
    const uint32_t k = sd.key_base + cell_key(g, ccx, ccy, ccz);
    key[i] = k;
    slot[i] = atomicAdd(count + k, 1u);
}

__global__ void k_pool_bcount(uint32_t N, Boundary<float> b, const uint32_t* __restrict__ bsid, const PoolScene* T,
                              uint32_t* __restrict__ key, uint32_t* __restrict__ slot, uint32_t* __restrict__ count)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const PoolScene& sd = T[bsid[i]];
    const uint32_t c = b.cell[i];
    const uint32_t k = sd.key_base + cell_key(sd.g, cell_x(c), cell_y(c), cell_z(c));
    key[i] = k;
    slot[i] = atomicAdd(count + k, 1u);
}

// The boundary points' half-precision copy for the list build's boundary
// cull (two points per 16-byte word, {x, y, z in the cell's modulo-3 frame},
// as the fluid's copy): boundary points do not move, so it is written once
// per re-layout.
__global__ void k_pool_boundary_half(uint32_t N, Boundary<float> b, const uint32_t* __restrict__ bsid, const PoolScene* T,
                                     uint4* __restrict__ posh)
{
    const uint32_t d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= N) return;
    const float h = T[bsid[d]].c.h;
    const P4<float> x = b.pos[d];
    __half* ph = reinterpret_cast<__half*>(posh) + (size_t)(d >> 1) * 8 + (d & 1);
    ph[0] = __float2half_rn(x.x);
    ph[2] = __float2half_rn(x.y);
    ph[4] = __float2half_rn(zframe3(x.z, cell_z(b.cell[d]), h));
}

// AkinciBoundaryModel::computeVolume (AkinciBoundayModel.cpp:11-40) per scene.
__global__ void k_pool_psi(uint32_t N, Boundary<float> b, const uint32_t* __restrict__ bsid, const PoolScene* T,
                           const uint32_t* __restrict__ bstarts)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const PoolScene& sd = T[bsid[i]];
    const Consts<float>& c = sd.c;
    float delta = 0.f;
    walk<float, 1>(sd.g, bstarts + sd.key_base, b.cell[i], xyz(b.pos[i]), c.h, 0, [&](uint32_t j, V3<float> s) {
        const V3<float> r = s - xyz(ldg4(b.pos + j));
        const float r2 = dot3(r, r);
        if (r2 <= c.cull2) delta += cubic_W(c, sqrtf(r2));
    });
    const float psi = 1.f / delta;
    b.psi[i] = psi;
    b.pos[i].w = c.density0 * psi;
}

// Pair-list build (k_build_lists per scene).  BLOCK threads per block, a
// register budget for MINB resident blocks per SM, and a shared candidate
// queue of qdepth entries per thread (dynamic shared memory, qdepth * BLOCK
// * 4 bytes) are tuning parameters; the lists do not depend on them (queued
// and re-walked candidates are accepted in the same walk order).
template <int BLOCK, int MINB, bool DIV0>
__global__ void __launch_bounds__(BLOCK, MINB) k_pool_build_lists(Fluid<float> f, const P4<float>* __restrict__ bpos,
                                                                         const uint32_t* __restrict__ sid, PoolScene* T,
                                                                         const uint32_t* __restrict__ cs,
                                                                         const uint32_t* __restrict__ bs, Lists<float> L,
                                                                         uint32_t qdepth)
{
    extern __shared__ uint32_t q[];
    const uint32_t i = blockIdx.x * BLOCK + threadIdx.x;
    uint32_t s = ~0u;
    unsigned long long contrib = 0ull;
    if (i < f.n) {
        const uint32_t k = sid[i];
        PoolScene& sd = T[k];
        if (sd.running) {
            float d = 0.f;
            uint32_t nn = 0;
            build_lists_one<float, true, DIV0>(i, f, bpos, sd.g, cs + sd.key_base, bs + sd.key_base, sd.c, sd.akinci, L,
                                               q, (uint32_t)BLOCK, qdepth, &d, &nn);
            if constexpr (DIV0) {
                // the divergence solve's first error pass (k_pool_errors<true,
                // true>'s arithmetic) from the sum the build just formed
                const Consts<float>& c = sd.c;
                const float dt = (float)sd.s.dt;
                const float inv0 = 1.f / c.density0;
                d = nn < 20u ? 0.f : (d < 0.f ? 0.f : d);
                f.div[i] = d;
                L.kbuf[i] = d * f.alpha[i] / (dt * f.rho[i]);
                contrib = error_contribution(d * inv0, sd);
                s = k;
            }
        }
    }
    if constexpr (DIV0) seg_add(s, contrib, T);
}

constexpr int kPoolForces = F_XSPH | F_STD_VISC | F_ART_VISC | F_SURFACE_TENSION | F_ADHESION;

// Surface normals of the scene's particles (SurfaceTensionAkinci.h:43-61)
// for the scenes with Akinci surface tension.
__global__ void __launch_bounds__(kBlock) k_pool_st_normals(Fluid<float> f, const uint32_t* __restrict__ sid,
                                                            const PoolScene* T, const uint32_t* __restrict__ cs)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= f.n) return;
    const PoolScene& sd = T[sid[i]];
    if (!sd.running || !(sd.c.force_flags & F_SURFACE_TENSION)) return;
    V3<float> ni = st_normal_sum<float, 1>(i, 0, f, sd.g, cs + sd.key_base, sd.c);
    ni = ni * (1.f * sd.c.h);
    f.normal[i] = P4<float>{ni.x, ni.y, ni.z, 0};
}

// Non-pressure forces of the scene (viscosity, surface tension, adhesion:
// k_npforce's walk and arithmetic, one lane per particle).
__global__ void __launch_bounds__(kBlock) k_pool_npforce(Fluid<float> f, const P4<float>* __restrict__ bpos,
                                                         const uint32_t* __restrict__ sid, const PoolScene* T,
                                                         const uint32_t* __restrict__ cs, const uint32_t* __restrict__ bs)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= f.n) return;
    const PoolScene& sd = T[sid[i]];
    const Consts<float>& c = sd.c;
    if (!sd.running || !(c.force_flags & kPoolForces)) return;
    const NPForces<float> s = npforce_sums<float, 1>(i, 0, f, bpos, sd.g, cs + sd.key_base, bs + sd.key_base, c,
                                                     sd.akinci, (float)sd.s.dt);
    npforce_apply(i, f, c, s);
}

// The list build's work at the current positions, for its FP32 roofline:
// candidates its walks visit (the 27 cells trimmed as the cull trims them;
// fluid, then boundary) and pairs within h, summed over running scenes into
// out[0..3] = fluid candidates, fluid pairs, boundary candidates, boundary
// pairs.  A diagnostic pass, not part of a step.
__global__ void k_pool_count_work(Fluid<float> f, const P4<float>* __restrict__ bpos, const uint32_t* __restrict__ sid,
                                  const PoolScene* T, const uint32_t* __restrict__ cs, const uint32_t* __restrict__ bs,
                                  unsigned long long* out)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long w[4] = {0ull, 0ull, 0ull, 0ull};
    if (i < f.n) {
        const PoolScene& sd = T[sid[i]];
        if (sd.running) {
            const V3<float> xi = xyz(f.pos[i]);
            const uint32_t pc = f.cell[i];
            walk<float, 1, true, true>(sd.g, cs + sd.key_base, pc, xi, sd.c.h, 0, [&](uint32_t j, V3<float> s) {
                const V3<float> r = s - xyz(ldg4(f.pos + j));
                ++w[0];
                if (dot3(r, r) <= sd.c.cull2) ++w[1];
            });
            if (sd.akinci)
                walk<float, 1>(sd.g, bs + sd.key_base, pc, xi, sd.c.h, 0, [&](uint32_t j, V3<float> s) {
                    const V3<float> r = s - xyz(ldg4(bpos + j));
                    ++w[2];
                    if (dot3(r, r) <= sd.c.cull2) ++w[3];
                });
        }
    }
    for (int q = 0; q < 4; ++q) {
        const unsigned long long v = warp_sum_u64(w[q]);
        if ((threadIdx.x & 31) == 0 && v) atomicAdd(out + q, v);
    }
}

// DFSPHSolver::updateTimeStep per scene: max of sqrt(|v + (a + g) dt|).
__global__ void k_pool_cfl_accum(Fluid<float> f, const uint32_t* __restrict__ sid, PoolScene* T)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t s = ~0u;
    float m = 0.f;
    if (i < f.n) {
        const uint32_t k = sid[i];
        const PoolScene& sd = T[k];
        if (sd.running) {
            const float dt = (float)sd.s.dt;
            const P4<float> v = f.vel[i], a = f.acc[i];
            const V3<float> cur = {v.x + (a.x + sd.c.gx) * dt, v.y + (a.y + sd.c.gy) * dt, v.z + (a.z + sd.c.gz) * dt};
            m = sqrtf(sqrtf(dot3(cur, cur)));
            s = k;
        }
    }
    const uint32_t s0 = __shfl_sync(0xffffffffu, s, 0);
    if (__all_sync(0xffffffffu, s == s0)) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
        if ((threadIdx.x & 31) == 0 && s0 != ~0u) atomicMax(&T[s0].vmax_bits, __float_as_uint(m));
    } else if (s != ~0u) {
        atomicMax(&T[s].vmax_bits, __float_as_uint(m));
    }
}

__global__ void k_pool_cfl_control(PoolScene* T, uint32_t S)
{
    for (uint32_t k = threadIdx.x; k < S; k += blockDim.x) {
        PoolScene& sd = T[k];
        if (!sd.running) continue;
        const double maxVel = fmax(0.1, (double)__uint_as_float(sd.vmax_bits));
        sd.vmax_bits = 0u;
        const double ts = sd.s.dt;
        const double cflTs = sd.lim.cflFactor * 0.4 * 2.0 * sd.lim.particleRadius / maxVel;
        double newTs;
        if (cflTs < ts) newTs = cflTs;
        else if (sd.s.iterations > 3) newTs = ts * 0.99;
        else newTs = ts * 1.001;
        newTs = fmax(newTs, sd.lim.minTs);
        newTs = fmin(newTs, sd.lim.maxTs);
        sd.s.dt = newTs;
        sd.s.maxVel = maxVel;
    }
}

__global__ void k_pool_predict_v_warm(Fluid<float> f, const uint32_t* __restrict__ sid, const PoolScene* T,
                                      float* __restrict__ kbuf)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= f.n) return;
    const PoolScene& sd = T[sid[i]];
    if (!sd.running) return;
    const Consts<float>& c = sd.c;
    const float dt = (float)sd.s.dt;
    P4<float> v = f.vel[i];
    const P4<float> a = f.acc[i];
    v.x = v.x + (a.x + c.gx) * dt; v.y = v.y + (a.y + c.gy) * dt; v.z = v.z + (a.z + c.gz) * dt;
    f.vel[i] = v;
    f.acc[i] = P4<float>{0, 0, 0, 0};
    const float t = -f.kappa[i] / f.rho[i];
    const float mx = t < -0.000000001f ? -0.000000001f : t;
    kbuf[i] = -mx / (dt * dt);
    f.kappa[i] = 0.f;
}

template <int BLOCK, int MINB, int MODE>
__global__ void __launch_bounds__(BLOCK, MINB) k_pool_correct(Fluid<float> f, const P4<float>* __restrict__ bpos,
                                                            const uint32_t* __restrict__ sid, const PoolScene* T,
                                                            const uint32_t* __restrict__ cs, const uint32_t* __restrict__ bs,
                                                            Lists<float> L)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= f.n) return;
    const PoolScene& sd = T[sid[i]];
    if (!sd.running || (MODE != 0 && !sd.loop_active)) return;
    const V3<float> sum = correct_sum_one<float, MODE>(i, f, bpos, sd.g, cs + sd.key_base, bs + sd.key_base, sd.c,
                                                       sd.akinci, L);
    correct_apply<float, MODE>(i, f, sd.c, (float)sd.s.dt, sum);
}

// DIV = false: DFSPHSolver::predictDensities; DIV = true:
// DFSPHSolver::computeDivergenceError.  Adds each scene's error sum.
template <int BLOCK, int MINB, bool DIV, bool INITIAL>
__global__ void __launch_bounds__(BLOCK, MINB) k_pool_errors(Fluid<float> f, const P4<float>* __restrict__ bpos,
                                                           const uint32_t* __restrict__ sid, PoolScene* T,
                                                           const uint32_t* __restrict__ cs, const uint32_t* __restrict__ bs,
                                                           Lists<float> L)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t s = ~0u;
    unsigned long long contrib = 0ull;
    if (i < f.n) {
        const uint32_t k = sid[i];
        PoolScene& sd = T[k];
        if (sd.running && (INITIAL || sd.loop_active)) {
            const Consts<float>& c = sd.c;
            const float dt = (float)sd.s.dt;
            const V3<float> vi = xyz(f.vel[i]);
            uint32_t nn;
            float d = velocity_div_one(i, f, bpos, sd.g, cs + sd.key_base, bs + sd.key_base, c, sd.akinci, L, vi, &nn);
            // the particle's relative error in FP32 (FP64 arithmetic is slow on
            // this part); its fixed-point quantum 2^-28 is still far coarser
            // than the FP32 rounding of an error of order 1e-3
            const float inv0 = 1.f / c.density0;
            float e;
            if (DIV) {
                d = nn < 20u ? 0.f : (d < 0.f ? 0.f : d);
                f.div[i] = d;
                L.kbuf[i] = d * f.alpha[i] / (dt * f.rho[i]);
                e = d * inv0;
            } else {
                const float rho = f.rho[i];
                float pred = rho + d * dt;
                pred = pred < c.density0 ? c.density0 : pred;
                f.pred[i] = pred;
                L.kbuf[i] = (pred - c.density0) * f.alpha[i] / ((dt * dt) * rho);
                e = (pred - c.density0) * inv0;
            }
            contrib = error_contribution(e, sd);
            s = k;
        }
    }
    seg_add(s, contrib, T);
}

// Loop control per scene after an error reduction (DFSPHSolver.cpp:325-401
// and :505-585): PHASE 0 density init, 1 density loop, 2 divergence init,
// 3 divergence loop.  Sets the "any scene still iterating" flag.
template <int PHASE>
__global__ void k_pool_control(PoolScene* T, uint32_t S, PoolCounters* pc, cudaGraphConditionalHandle cond)
{
    unsigned any = 0;
    for (uint32_t k = threadIdx.x; k < S; k += blockDim.x) {
        PoolScene& sd = T[k];
        const unsigned long long acc = sd.acc;
        const uint32_t bad = sd.bad;
        sd.acc = 0ull;
        sd.bad = 0u;
        if (!sd.running) { sd.loop_active = 0; continue; }
        double avg = sd.n ? (double)acc / kFixScale / (double)sd.n : 0.0;
        // a NaN / Inf error makes the average NaN (the loop then stops at its
        // minimum iterations, as the reference's NaN comparisons do), an
        // error above the clamp makes it +Inf (the loop runs to its cap)
        if (bad & 1u) {
            avg = __longlong_as_double(0x7ff8000000000000ll);
            sd.s.status |= ST_NONFINITE;
        } else if (bad & 2u) {
            avg = __longlong_as_double(0x7ff0000000000000ll);
            sd.s.status |= ST_DIVERGED;
        }
        const LoopLimits& lim = sd.lim;
        unsigned act;
        if (PHASE == 0) {
            sd.s.iterations = 0;
            sd.s.avgDensError = avg;
            act = (lim.minIt > 0u) && (lim.maxIt > 0u);
        } else if (PHASE == 2) {
            sd.s.iterationsV = 0;
            sd.s.avgDivError = avg;
            act = (lim.minItV > 0u) && (lim.maxIt > 0u);
        } else {
            if (!sd.loop_active) continue;
            if (PHASE == 1) {
                const unsigned it = ++sd.s.iterations;
                sd.s.avgDensError = avg;
                act = ((avg > lim.maxError) || (it < lim.minIt)) && (it < lim.maxIt);
                if (!act) {
                    sd.s.sumIterations += it;
                    if (it >= lim.maxIt && avg > lim.maxError) sd.s.status |= ST_ITER_CAP;
                }
            } else {
                const unsigned it = ++sd.s.iterationsV;
                const double lim_v = lim.maxErrorV / sd.s.dt;
                sd.s.avgDivError = avg;
                act = ((avg > lim_v) || (it < lim.minItV)) && (it < lim.maxIt);
                if (!act) {
                    sd.s.sumIterationsV += it;
                    if (it >= lim.maxIt && avg > lim_v) sd.s.status |= ST_ITER_CAP_V;
                }
            }
        }
        sd.loop_active = act;
        any |= act;
    }
    any = __syncthreads_or(any);
    if (threadIdx.x == 0) {
        if (PHASE == 1 || PHASE == 3) {
            if (PHASE == 1) pc->body_d += 1;
            else pc->body_v += 1;
        }
        pc->any = any;
        if (cond) cudaGraphSetConditional(cond, any);
    }
}

// Each scene's running flag, for a poll that copies S bytes.
__global__ void k_pool_running(const PoolScene* __restrict__ T, uint32_t S, uint8_t* __restrict__ out)
{
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < S; k += gridDim.x * blockDim.x) out[k] = T[k].running ? 1 : 0;
}

__global__ void k_pool_finish(PoolScene* T, uint32_t S)
{
    for (uint32_t k = threadIdx.x; k < S; k += blockDim.x) {
        PoolScene& sd = T[k];
        if (!sd.running) continue;
        sd.s.time = sd.s.time + sd.s.dt;
        sd.s.steps += 1;
        sd.steps_left -= 1;
        // a scene whose state turned NaN / Inf is retired after this step:
        // polls report it done, its status carries SPH_STATUS_NONFINITE
        if (sd.s.status & ST_NONFINITE) sd.steps_left = 0;
        sd.running = sd.steps_left > 0;
    }
}

// ===========================================================================
// Host side
// ===========================================================================

struct PoolEntry {
    int id = -1;
    sph_scene_desc d{};
    bool staged = false;          // points (x, v, boundary) in the staging arena until resident
    size_t ox = 0, ov = 0, ob = 0;  // their offsets there
    bool restored = false;        // staged from a snapshot: raw device arrays at ox, solver scalars
    DevScalars snap_s{};
    unsigned n = 0, nb = 0, steps = 0;
    GridPlan plan;
    PoolScene t{};                // last known device entry (layout fields kept by the host)
    bool resident = false;
    bool removed = false;
};

// A scene snapshot: this header, then the scene's device arrays as stored
// (sorted order; cell-relative FP32 positions with their packed cells), each
// starting on a 16-byte boundary.
struct SnapHeader {
    char magic[8];          // "SPHPSNP1"
    uint32_t version, desc_size, scalars_size, n, nb, steps_left;
    int32_t o[3], nn[3];    // the scene's grid box
    uint64_t bytes;         // header and arrays
    sph_scene_desc d;
    DevScalars s;
};
constexpr uint32_t kSnapVersion = 1;

// Byte offsets of the raw arrays after the header: fluid pos, vel (16 B
// each), kappa, kappav, pred, cell, id (4 B), boundary pos (16 B), cell, id
// (4 B).  out[10] = total bytes of the arrays.
inline void snap_layout(size_t n, size_t nb, size_t out[11])
{
    const size_t sz[10] = {16 * n, 16 * n, 4 * n, 4 * n, 4 * n, 4 * n, 4 * n, 16 * nb, 4 * nb, 4 * nb};
    size_t off = 0;
    for (int k = 0; k < 10; ++k) {
        out[k] = off;
        off += (sz[k] + 15) / 16 * 16;
    }
    out[10] = off;
}

class Pool {
public:
    struct Tune { int build_block = 256, build_occ = 768, queue = 48, solver_block = 128, solver_occ = 1024, scan_per = 16; };
    std::string err;

    ~Pool()
    {
        for (auto& e : gexec_) if (e) cudaGraphExecDestroy(e);
        for (auto& q : pending_) { cudaEventDestroy(q.a); cudaEventDestroy(q.b); }
        for (auto& q : tpending_) { cudaEventDestroy(q.a); cudaEventDestroy(q.b); }
        for (auto e : events_) cudaEventDestroy(e);
        for (auto e : tev_) if (e) cudaEventDestroy(e);
        if (st_) cudaStreamDestroy(st_);
        if (st2_) cudaStreamDestroy(st2_);
        if (up_) { cudaStreamSynchronize(up_); cudaStreamDestroy(up_); }
        if (h_box_) cudaFreeHost(h_box_);
        if (h_pc_) cudaFreeHost(h_pc_);
        if (h_run_) cudaFreeHost(h_run_);
    }

    void fail(const std::string& m) { err = m; }

    int create(const sph_pool_desc& d)
    {
        pd_ = d;
        if (d.max_particles == 0 || d.max_scenes == 0 || d.max_keys == 0) { fail("empty pool capacity"); return SPH_ERR_INVALID; }
        if (d.max_particles >= (1ull << 31) || d.max_boundary >= (1ull << 31) || d.max_keys >= (1ull << 31)) {
            fail("pool capacity above 2^31");
            return SPH_ERR_CAPACITY;
        }
        kmax_ = d.neighbor_list_max > 0 ? (uint32_t)d.neighbor_list_max : 64u;
        SPH_CUDA(cudaStreamCreateWithFlags(&st_, cudaStreamNonBlocking));
        SPH_CUDA(cudaStreamCreateWithFlags(&st2_, cudaStreamNonBlocking));
        SPH_CUDA(cudaStreamCreateWithFlags(&up_, cudaStreamNonBlocking));
        SPH_CUDA(box_.alloc(12 * kBoxBlocks));
        SPH_CUDA(cudaMallocHost((void**)&h_box_, 12 * kBoxBlocks * sizeof(double)));
        ls_ = st_;
        SPH_CUDA(cudaMallocHost((void**)&h_pc_, sizeof(PoolCounters)));
        SPH_CUDA(cudaMallocHost((void**)&h_run_, std::max<size_t>(d.max_scenes, 1)));
        const size_t P = d.max_particles, B = std::max<size_t>(d.max_boundary, 1), K = d.max_keys;
        for (int k = 0; k < 2; ++k) {
            SPH_CUDA(pos_[k].alloc(P)); SPH_CUDA(vel_[k].alloc(P)); SPH_CUDA(kappa_[k].alloc(P));
            SPH_CUDA(kappav_[k].alloc(P)); SPH_CUDA(pred_[k].alloc(P)); SPH_CUDA(cell_[k].alloc(P)); SPH_CUDA(id_[k].alloc(P));
            SPH_CUDA(bpos_[k].alloc(B)); SPH_CUDA(bcell_[k].alloc(B)); SPH_CUDA(bid_[k].alloc(B));
        }
        SPH_CUDA(acc_.alloc(P)); SPH_CUDA(rho_.alloc(P)); SPH_CUDA(alpha_.alloc(P)); SPH_CUDA(div_.alloc(P));
        SPH_CUDA(press_.alloc(P)); SPH_CUDA(kbuf_.alloc(P)); SPH_CUDA(sid_.alloc(P)); SPH_CUDA(bsid_.alloc(B));
        SPH_CUDA(bpsi_.alloc(B)); SPH_CUDA(dummy4_.alloc(1)); SPH_CUDA(normal_.alloc(P));
        SPH_CUDA(pairs_.alloc(P * kmax_)); SPH_CUDA(lcount_.alloc(P)); SPH_CUDA(bgrad_.alloc(P));
        SPH_CUDA(posh_.alloc(P / 2 + 2));  // particle pairs, the last one whole, and a spare word for the cull
        SPH_CUDA(cudaMemsetAsync(posh_.p, 0, (P / 2 + 2) * sizeof(uint4), st_));
        SPH_CUDA(bposh_.alloc(B / 2 + 2));
        SPH_CUDA(cudaMemsetAsync(bposh_.p, 0, (B / 2 + 2) * sizeof(uint4), st_));
        const size_t M = std::max(P, B);
        SPH_CUDA(key_.alloc(M)); SPH_CUDA(slot_.alloc(M)); SPH_CUDA(tmp_.alloc(M));
        SPH_CUDA(count_.alloc(K)); SPH_CUDA(starts_.alloc(K + 1)); SPH_CUDA(bstarts_.alloc(K + 1));
        SPH_CUDA(tile_sums_.alloc((K + kScanThreads * 4 - 1) / (kScanThreads * 4) + 1));
        SPH_CUDA(cudaFuncSetAttribute(k_pool_build_lists<256, 3, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      64 * 256 * (int)sizeof(uint32_t)));
        SPH_CUDA(cudaFuncSetAttribute(k_pool_build_lists<256, 4, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      64 * 256 * (int)sizeof(uint32_t)));
        SPH_CUDA(cudaFuncSetAttribute(k_pool_build_lists<256, 3, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      64 * 256 * (int)sizeof(uint32_t)));
        SPH_CUDA(cudaFuncSetAttribute(k_pool_build_lists<256, 4, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      64 * 256 * (int)sizeof(uint32_t)));
        SPH_CUDA(cudaMemsetAsync(count_.p, 0, K * sizeof(uint32_t), st_));
        SPH_CUDA(table_.alloc(d.max_scenes));
        SPH_CUDA(run_.alloc(d.max_scenes));
        SPH_CUDA(seg_a_.alloc(d.max_scenes)); SPH_CUDA(seg_b_.alloc(d.max_scenes)); SPH_CUDA(seg_n_.alloc(d.max_scenes));
        SPH_CUDA(pc_.alloc(1));
        SPH_CUDA(cudaMemsetAsync(pc_.p, 0, sizeof(PoolCounters), st_));
        SPH_CUDA(cudaStreamSynchronize(st_));
        return SPH_OK;
    }

    // Admission (applied at the next step).  SPH_ERR_CAPACITY: does not fit now.
    int add(const sph_scene_desc& d, const double* x, const double* v, unsigned n, const double* b, unsigned nb,
            unsigned steps, int* id)
    {
        if (d.simulation_method != SPH_DFSPH || d.boundary_method != SPH_BOUNDARY_AKINCI) {
            fail("the pool runs DFSPH scenes with Akinci boundaries");
            return SPH_ERR_UNSUPPORTED;
        }
        if (n == 0 || !x) { fail("no fluid particles"); return SPH_ERR_INVALID; }
        PoolEntry e;
        e.d = d;
        e.n = n;
        e.nb = nb;
        e.steps = steps;
        double hh, mass;
        scene_constants<float>(d, &e.t.c, &e.t.lim, &hh, &mass);
        // capacity check against everything resident or pending (grid keys
        // once the scene's box is known, below)
        uint64_t P = 0, B = 0, K = 0;
        unsigned S = 0;
        for (auto& q : entries_) {
            if (q.removed) continue;
            P += q.n; B += q.nb; K += q.plan.nkeys; ++S;
        }
        if (P + n > pd_.max_particles || B + nb > pd_.max_boundary || S + 1 > pd_.max_scenes) {
            fail("pool full");
            return SPH_ERR_CAPACITY;
        }
        // the points go straight from the caller's arrays into the device
        // staging arena on the upload stream (no host copy; a step running on
        // the pool's stream meanwhile is not waited for); the copy is complete
        // when this returns, so the caller may reuse its arrays
        const size_t nx = 3 * (size_t)n, nbv = 3 * (size_t)nb, need = 2 * nx + nbv;
        if (int grc = reserve_arena(need)) return grc;
        e.ox = arena_used_;
        e.ov = e.ox + nx;
        e.ob = e.ov + nx;
        double* a = arena_.p;
        cudaError_t ce = cudaMemcpyAsync(a + e.ox, x, nx * sizeof(double), cudaMemcpyHostToDevice, up_);
        if (ce == cudaSuccess)
            ce = v ? cudaMemcpyAsync(a + e.ov, v, nx * sizeof(double), cudaMemcpyHostToDevice, up_)
                   : cudaMemsetAsync(a + e.ov, 0, nx * sizeof(double), up_);
        if (ce == cudaSuccess && nb) ce = cudaMemcpyAsync(a + e.ob, b, nbv * sizeof(double), cudaMemcpyHostToDevice, up_);
        // the points' bounding box, formed on the device from the staged copy
        const unsigned gx = std::min<unsigned>(kBoxBlocks, blocks(n, 256));
        const unsigned gb = nb ? std::min<unsigned>(kBoxBlocks, blocks(nb, 256)) : 0u;
        if (ce == cudaSuccess) {
            k_point_box<<<gx, 256, 0, up_>>>(a + e.ox, n, box_.p);
            if (gb) k_point_box<<<gb, 256, 0, up_>>>(a + e.ob, nb, box_.p + 6 * kBoxBlocks);
            ce = cudaGetLastError();
        }
        if (ce == cudaSuccess) ce = cudaMemcpyAsync(h_box_, box_.p, 12 * kBoxBlocks * sizeof(double), cudaMemcpyDeviceToHost, up_);
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(up_);
        if (ce != cudaSuccess) {
            fail(std::string("staging a scene: ") + cudaGetErrorString(ce));
            return SPH_ERR_CUDA;
        }
        double box[6] = {1e300, 1e300, 1e300, -1e300, -1e300, -1e300};
        auto merge = [&](const double* part, unsigned nblk) {
            for (unsigned q = 0; q < nblk; ++q)
                for (int k = 0; k < 3; ++k) {
                    box[k] = std::min(box[k], part[6 * q + k]);
                    box[3 + k] = std::max(box[3 + k], part[6 * q + 3 + k]);
                }
        };
        merge(h_box_, gx);
        merge(h_box_ + 6 * kBoxBlocks, gb);
        // the walls bound a pooled scene: two cells beyond its points, no
        // proportional margin (a box just over 32 cells wide would double
        // each Morton axis of its key space)
        int rc = grid_plan(d, PointSpan(x, 3 * (size_t)n), PointSpan(b, 3 * (size_t)nb), true, PointSpan(nullptr, 0), hh,
                           &e.plan, &err, 0.0, false, box);
        if (rc) return rc;
        if (K + e.plan.nkeys > pd_.max_keys) {
            fail("pool full");
            return SPH_ERR_CAPACITY;
        }
        arena_used_ += need;
        e.staged = true;
        e.id = next_id_++;
        *id = e.id;
        entries_.push_back(std::move(e));
        dirty_ = true;
        return SPH_OK;
    }

    // Room for `need` more doubles in the staging arena (grows by doubling;
    // the pending scenes' data moves to the new arena).
    int reserve_arena(size_t need)
    {
        if (arena_used_ + need <= arena_.n) return SPH_OK;
        DevBuf<double> bigger;
        SPH_CUDA(bigger.alloc(std::max(arena_used_ + need, 2 * arena_.n)));
        if (arena_used_)
            SPH_CUDA(cudaMemcpyAsync(bigger.p, arena_.p, arena_used_ * sizeof(double), cudaMemcpyDeviceToDevice, up_));
        SPH_CUDA(cudaStreamSynchronize(up_));
        std::swap(arena_.p, bigger.p);
        std::swap(arena_.n, bigger.n);
        return SPH_OK;
    }

    // A resident scene's snapshot (see sph_pool_snapshot).
    int snapshot(int id, void* buf, unsigned long long cap, unsigned long long* size)
    {
        PoolEntry* e = find(id);
        if (!e || !e->resident) { fail("scene is not resident"); return SPH_ERR_INVALID; }
        size_t L[11];
        snap_layout(e->n, e->nb, L);
        const size_t need = sizeof(SnapHeader) + L[10];
        *size = need;
        if (!buf) return SPH_OK;
        if (cap < need) { fail("snapshot buffer too small"); return SPH_ERR_CAPACITY; }
        SPH_CUDA(cudaStreamSynchronize(st_));
        PoolScene t;
        SPH_CUDA(cudaMemcpy(&t, table_.p + slot_of(id), sizeof t, cudaMemcpyDeviceToHost));
        SnapHeader h;
        std::memset(&h, 0, sizeof h);
        std::memcpy(h.magic, "SPHPSNP1", 8);
        h.version = kSnapVersion;
        h.desc_size = sizeof(sph_scene_desc);
        h.scalars_size = sizeof(DevScalars);
        h.n = e->n;
        h.nb = e->nb;
        h.steps_left = t.steps_left;
        for (int k = 0; k < 3; ++k) { h.o[k] = e->plan.o[k]; h.nn[k] = e->plan.nn[k]; }
        h.bytes = need;
        h.d = e->d;
        h.s = t.s;
        char* out = static_cast<char*>(buf);
        std::memcpy(out, &h, sizeof h);
        char* a = out + sizeof h;
        const size_t n = e->n, nb = e->nb, pb = t.pbase, bb = t.bbase;
        const void* src[10] = {pos_[cur_].p + pb, vel_[cur_].p + pb, kappa_[cur_].p + pb, kappav_[cur_].p + pb,
                               pred_[cur_].p + pb, cell_[cur_].p + pb, id_[cur_].p + pb, bpos_[bcur_].p + bb,
                               bcell_[bcur_].p + bb, bid_[bcur_].p + bb};
        const size_t sz[10] = {16 * n, 16 * n, 4 * n, 4 * n, 4 * n, 4 * n, 4 * n, 16 * nb, 4 * nb, 4 * nb};
        for (int k = 0; k < 10; ++k)
            if (sz[k]) SPH_CUDA(cudaMemcpyAsync(a + L[k], src[k], sz[k], cudaMemcpyDeviceToHost, st_));
        SPH_CUDA(cudaStreamSynchronize(st_));
        return SPH_OK;
    }

    // A scene admitted from a snapshot (see sph_pool_restore).
    int restore(const void* buf, unsigned long long size, unsigned steps, int* id)
    {
        SnapHeader h;
        if (!buf || size < sizeof h) { fail("not a scene snapshot (too short)"); return SPH_ERR_INVALID; }
        std::memcpy(&h, buf, sizeof h);
        if (std::memcmp(h.magic, "SPHPSNP1", 8) != 0 || h.version != kSnapVersion || h.desc_size != sizeof(sph_scene_desc) ||
            h.scalars_size != sizeof(DevScalars)) {
            fail("not a scene snapshot of this library version");
            return SPH_ERR_INVALID;
        }
        size_t L[11];
        snap_layout(h.n, h.nb, L);
        if (h.n == 0 || h.bytes != size || size != sizeof h + L[10]) { fail("scene snapshot of the wrong size"); return SPH_ERR_INVALID; }
        PoolEntry e;
        e.d = h.d;
        e.n = h.n;
        e.nb = h.nb;
        e.steps = steps ? steps : h.steps_left;
        double hh, mass;
        scene_constants<float>(e.d, &e.t.c, &e.t.lim, &hh, &mass);
        int rc = grid_plan_box(h.o, h.nn, &e.plan, &err);
        if (rc) return rc;
        uint64_t P = 0, B = 0, K = 0;
        unsigned S = 0;
        for (auto& q : entries_) {
            if (q.removed) continue;
            P += q.n; B += q.nb; K += q.plan.nkeys; ++S;
        }
        if (P + e.n > pd_.max_particles || B + e.nb > pd_.max_boundary || K + e.plan.nkeys > pd_.max_keys ||
            S + 1 > pd_.max_scenes) {
            fail("pool full");
            return SPH_ERR_CAPACITY;
        }
        const size_t need = (L[10] + 7) / 8;
        if (int grc = reserve_arena(need)) return grc;
        e.ox = arena_used_;
        SPH_CUDA(cudaMemcpyAsync(arena_.p + e.ox, static_cast<const char*>(buf) + sizeof h, L[10], cudaMemcpyHostToDevice, up_));
        SPH_CUDA(cudaStreamSynchronize(up_));
        arena_used_ += need;
        e.staged = true;
        e.restored = true;
        e.snap_s = h.s;
        e.id = next_id_++;
        *id = e.id;
        entries_.push_back(std::move(e));
        dirty_ = true;
        return SPH_OK;
    }

    int remove(int id)
    {
        for (auto& e : entries_)
            if (e.id == id && !e.removed) {
                e.removed = true;
                dirty_ = true;
                return SPH_OK;
            }
        fail("unknown scene id");
        return SPH_ERR_INVALID;
    }

    int step(int nsteps)
    {
        // nsteps == 0 applies pending admissions and removals only
        if (nsteps == 0 && dirty_) return relayout();
        for (int k = 0; k < nsteps; ++k) {
            if (dirty_) {
                const int rc = relayout();
                if (rc) return rc;
            }
            if (S_ == 0) return SPH_OK;
            Phase ph(phases_, "Step computation", st_, false, prof_ && tune_left_ == 0);
            const int rc = tune_left_ > 0 ? tuning_step() : graph_ ? graph_step() : one_step();
            if (rc) return rc;
        }
        return SPH_OK;
    }

    int set_graph(int on) { graph_ = on != 0; return SPH_OK; }

    // ---- autotuner --------------------------------------------------------
    // Candidates: pair-list build shape (block, register budget) x queue
    // depth, solver-pass shape (block, register budget), scan width.  Each
    // family's kernels are timed separately (CUDA events) over 2 x 12
    // host-driven steps that cycle through the candidates, and the fastest
    // candidate of each family is kept.  Tuning steps are ordinary steps of
    // every resident scene: no candidate changes any result.  The choice is
    // cached per GPU model, particle-count bucket (next power of two) and list
    // width in a text file (SPH_GB300_TUNE_FILE, default
    // ~/.cache/sph_gb300_tune.txt) and re-measured only for a new bucket.
    struct Shape { int block, occ; };
    static constexpr Shape kBuild[4] = {{128, 896}, {128, 1024}, {256, 768}, {256, 1024}};
    static constexpr int kQD[3] = {40, 48, 56};
    static constexpr Shape kSolver[6] = {{128, 1024}, {128, 1536}, {128, 2048}, {256, 1024}, {256, 1536}, {256, 2048}};
    static constexpr int kSW[3] = {4, 8, 16};
    static constexpr int kNBuild = 12, kNSolver = 6, kNScan = 3;
    static constexpr int kTuneSteps = 2 * kNBuild;

    static bool valid(const Tune& t)
    {
        bool b = false, s = false;
        for (const Shape& q : kBuild) b |= q.block == t.build_block && q.occ == t.build_occ;
        for (const Shape& q : kSolver) s |= q.block == t.solver_block && q.occ == t.solver_occ;
        const bool qd = t.queue >= 8 && t.queue <= 64 && t.queue % 8 == 0;
        const bool w = t.scan_per == 4 || t.scan_per == 8 || t.scan_per == 16;
        return b && s && qd && w;
    }
    static Tune candidate(int bc, int sc, int wc)
    {
        return Tune{kBuild[bc / 3].block, kBuild[bc / 3].occ, kQD[bc % 3], kSolver[sc].block, kSolver[sc].occ, kSW[wc]};
    }

    int set_autotune(int mode)
    {
        if (mode < 0 || mode > 2) { fail("autotune mode is 0, 1 or 2"); return SPH_ERR_INVALID; }
        tune_mode_ = mode;
        tune_bucket_ = 0;  // decide again at the next re-layout
        if (mode == 0) tune_left_ = 0;
        dirty_ = dirty_ || (mode != 0 && S_ > 0);
        return SPH_OK;
    }

    int set_tuning(const sph_pool_tuning& t)
    {
        const Tune v{t.build_block, t.build_occupancy, t.queue_depth, t.solver_block, t.solver_occupancy, t.scan_width};
        if (!valid(v)) {
            fail("tuning values outside the supported shapes");
            return SPH_ERR_INVALID;
        }
        tune_ = v;
        tune_source_ = 0;
        tune_mode_ = 0;
        tune_left_ = 0;
        drop_graphs();
        return SPH_OK;
    }

    void get_tuning(sph_pool_tuning* t) const
    {
        t->build_block = tune_.build_block;
        t->build_occupancy = tune_.build_occ;
        t->queue_depth = tune_.queue;
        t->solver_block = tune_.solver_block;
        t->solver_occupancy = tune_.solver_occ;
        t->scan_width = tune_.scan_per;
        t->source = tune_source_;
        t->steps_left = tune_left_;
    }

    const std::string& tuning_log() const { return tune_log_; }

    static void tune_family(const char* name, int* fam, int* sub)
    {
        if (!std::strcmp(name, "k_pool_build_lists")) { *fam = 0; *sub = 0; }
        else if (!std::strcmp(name, "k_pool_correct")) { *fam = 1; *sub = 0; }
        else if (!std::strcmp(name, "k_pool_errors_density")) { *fam = 1; *sub = 1; }
        else if (!std::strcmp(name, "k_pool_errors_div")) { *fam = 1; *sub = 2; }
        else if (!std::strcmp(name, "k_scan_tiles")) { *fam = 2; *sub = 0; }
        else if (!std::strcmp(name, "k_scan_add")) { *fam = 2; *sub = 1; }
    }

    std::string tune_key() const
    {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceProp prop;
        std::memset(&prop, 0, sizeof prop);
        cudaGetDeviceProperties(&prop, dev);
        char k[320];
        std::snprintf(k, sizeof k, "%s|sm%d%d|n%llu|k%u", prop.name, prop.major, prop.minor,
                      (unsigned long long)tune_bucket_, kmax_);
        std::string out = k;
        for (auto& ch : out) if (ch == ' ') ch = '_';
        return out;
    }

    static std::string tune_path()
    {
        const char* e = std::getenv("SPH_GB300_TUNE_FILE");
        if (e && *e) return e;
        const char* home = std::getenv("HOME");
        if (!home || !*home) return "";
        std::string d = std::string(home) + "/.cache";
        mkdir(d.c_str(), 0755);
        return d + "/sph_gb300_tune.txt";
    }

    bool cache_lookup(const std::string& key, Tune* t) const
    {
        const std::string path = tune_path();
        if (path.empty()) return false;
        FILE* fp = std::fopen(path.c_str(), "r");
        if (!fp) return false;
        char line[512], k[400];
        Tune v;
        bool hit = false;
        while (std::fgets(line, sizeof line, fp))
            if (std::sscanf(line, "%399s %d %d %d %d %d %d", k, &v.build_block, &v.build_occ, &v.queue, &v.solver_block,
                            &v.solver_occ, &v.scan_per) == 7 && key == k && valid(v)) {
                *t = v;
                hit = true;
            }
        std::fclose(fp);
        return hit;
    }

    void cache_store(const std::string& key, const Tune& t) const
    {
        const std::string path = tune_path();
        if (path.empty()) return;
        FILE* fp = std::fopen(path.c_str(), "a");
        if (!fp) return;
        std::fprintf(fp, "%s %d %d %d %d %d %d\n", key.c_str(), t.build_block, t.build_occ, t.queue, t.solver_block,
                     t.solver_occ, t.scan_per);
        std::fclose(fp);
    }

    // After a re-layout: use the cached choice for this bucket, or measure.
    void tune_after_relayout()
    {
        if (tune_mode_ == 0 || N_ == 0) return;
        unsigned long long b = 1;
        while (b < N_) b <<= 1;
        if (b == tune_bucket_ && tune_mode_ == 1) return;
        tune_bucket_ = b;
        Tune t;
        if (tune_mode_ == 1 && cache_lookup(tune_key(), &t)) {
            tune_ = t;
            tune_source_ = 1;
            return;
        }
        std::memset(tacc_ms_, 0, sizeof tacc_ms_);
        std::memset(tacc_n_, 0, sizeof tacc_n_);
        tune_left_ = kTuneSteps;
        tune_step_ = 0;
    }

    int tuning_step()
    {
        const int t = tune_step_++;
        const int bc = t % kNBuild, sc = t % kNSolver, wc = (t / kNSolver) % kNScan;
        cand_[0] = bc; cand_[1] = sc; cand_[2] = wc;
        tune_ = candidate(bc, sc, wc);
        tuning_ = true;
        const int rc = one_step();
        tuning_ = false;
        SPH_CUDA(cudaStreamSynchronize(st_));
        for (auto& q : tpending_) {
            float ms = 0.f;
            if (rc == SPH_OK) SPH_CUDA(cudaEventElapsedTime(&ms, q.a, q.b));
            tacc_ms_[q.fam][cand_[q.fam]][q.sub] += ms;
            tacc_n_[q.fam][cand_[q.fam]][q.sub] += 1;
            events_.push_back(q.a);
            events_.push_back(q.b);
        }
        tpending_.clear();
        if (rc) return rc;
        if (--tune_left_ == 0) finish_tuning();
        return SPH_OK;
    }

    void finish_tuning()
    {
        const int ncand[3] = {kNBuild, kNSolver, kNScan};
        int best[3] = {2 * 3 + 1, 0, 2};
        char line[160];
        tune_log_.clear();
        for (int fam = 0; fam < 3; ++fam) {
            double bestc = 1e300;
            for (int c = 0; c < ncand[fam]; ++c) {
                double cost = 0.0;
                bool any = false;
                for (int sub = 0; sub < 3; ++sub)
                    if (tacc_n_[fam][c][sub]) { cost += tacc_ms_[fam][c][sub] / tacc_n_[fam][c][sub]; any = true; }
                if (!any) continue;
                if (fam == 0)
                    std::snprintf(line, sizeof line, "build block %d occupancy %d queue %d: %.4f ms\n", kBuild[c / 3].block,
                                  kBuild[c / 3].occ, kQD[c % 3], cost);
                else if (fam == 1)
                    std::snprintf(line, sizeof line, "solver block %d occupancy %d: %.4f ms\n", kSolver[c].block,
                                  kSolver[c].occ, cost);
                else
                    std::snprintf(line, sizeof line, "scan width %d: %.4f ms\n", kSW[c], cost);
                tune_log_ += line;
                if (cost < bestc) { bestc = cost; best[fam] = c; }
            }
        }
        tune_ = candidate(best[0], best[1], best[2]);
        tune_source_ = 2;
        if (tune_mode_ == 2) tune_mode_ = 1;
        cache_store(tune_key(), tune_);
        drop_graphs();
    }

    void drop_graphs()
    {
        for (auto& e : gexec_) if (e) { cudaGraphExecDestroy(e); e = nullptr; }
    }
    int set_profiling(int on) { prof_ = on != 0; return SPH_OK; }

    // Phase times (CUDA events, profiling on) since the last call.
    int phase_profile(char* buf, size_t len)
    {
        SPH_CUDA(cudaStreamSynchronize(st_));
        const int n = phases_.report(buf, len);
        if (n < 0) { fail(cudaGetErrorString((cudaError_t)-n)); return SPH_ERR_CUDA; }
        return n;
    }
    // a named phase of a host-driven step (nothing while capturing or tuning)
    Phase phase(const char* name) { return Phase(phases_, name, ls_, capturing_, prof_ && counting_ && !tuning_); }

    // "name launches total_ms" per kernel for the host-driven steps timed
    // since the previous call.
    int profile(char* buf, size_t len)
    {
        SPH_CUDA(cudaStreamSynchronize(st_));
        std::vector<std::string> names;
        std::vector<double> ms;
        std::vector<unsigned long long> cnt;
        for (auto& q : pending_) {
            float t = 0.f;
            SPH_CUDA(cudaEventElapsedTime(&t, q.a, q.b));
            size_t k = 0;
            while (k < names.size() && names[k] != q.name) ++k;
            if (k == names.size()) { names.push_back(q.name); ms.push_back(0.0); cnt.push_back(0); }
            ms[k] += t;
            cnt[k] += 1;
            events_.push_back(q.a);
            events_.push_back(q.b);
        }
        pending_.clear();
        std::string outs;
        char line[256];
        for (size_t k = 0; k < names.size(); ++k) {
            std::snprintf(line, sizeof line, "%s %llu %.6f\n", names[k].c_str(), cnt[k], ms[k]);
            outs += line;
        }
        if (buf && len) {
            std::strncpy(buf, outs.c_str(), len - 1);
            buf[len - 1] = 0;
        }
        return (int)outs.size();
    }

    // nsteps steps bracketed by CUDA events on the pool's stream.
    int step_timed(int nsteps, float* ms)
    {
        if (!tev_[0]) {
            SPH_CUDA(cudaEventCreate(&tev_[0]));
            SPH_CUDA(cudaEventCreate(&tev_[1]));
        }
        if (dirty_) {
            const int rc = relayout();
            if (rc) return rc;
        }
        SPH_CUDA(cudaEventRecord(tev_[0], st_));
        const int rc = step(nsteps);
        if (rc) return rc;
        SPH_CUDA(cudaEventRecord(tev_[1], st_));
        SPH_CUDA(cudaEventSynchronize(tev_[1]));
        SPH_CUDA(cudaEventElapsedTime(ms, tev_[0], tev_[1]));
        return SPH_OK;
    }

    // Stored pairs and overflowing particles of the running scenes' lists.
    int list_pairs(unsigned long long* pairs, unsigned* overflow)
    {
        DevBuf<unsigned long long> o;
        SPH_CUDA(o.alloc(2));
        SPH_CUDA(cudaMemsetAsync(o.p, 0, 2 * sizeof(unsigned long long), st_));
        if (N_) k_list_stats<<<blocks(N_, 256), 256, 0, st_>>>(N_, lcount_.p, kmax_, o.p);
        SPH_CUDA(cudaGetLastError());
        unsigned long long h[2];
        SPH_CUDA(cudaMemcpyAsync(h, o.p, sizeof h, cudaMemcpyDeviceToHost, st_));
        SPH_CUDA(cudaStreamSynchronize(st_));
        *pairs = h[0];
        *overflow = (unsigned)h[1];
        return SPH_OK;
    }

    int count_work(unsigned long long out[4])
    {
        DevBuf<unsigned long long> o;
        SPH_CUDA(o.alloc(4));
        SPH_CUDA(cudaMemsetAsync(o.p, 0, 4 * sizeof(unsigned long long), st_));
        if (N_)
            k_pool_count_work<<<blocks(N_, 256), 256, 0, st_>>>(F(cur_), bpos_[bcur_].p, sid_.p, table_.p, starts_.p,
                                                                 bstarts_.p, o.p);
        SPH_CUDA(cudaGetLastError());
        SPH_CUDA(cudaMemcpyAsync(out, o.p, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st_));
        SPH_CUDA(cudaStreamSynchronize(st_));
        return SPH_OK;
    }

    int sync()
    {
        SPH_CUDA(cudaStreamSynchronize(st_));
        return SPH_OK;
    }

    // Statistics of one scene; *done = its steps have completed.
    int query(int id, sph_stats* out, int* done)
    {
        PoolEntry* e = find(id);
        if (!e) { fail("unknown scene id"); return SPH_ERR_INVALID; }
        std::memset(out, 0, sizeof *out);
        if (!e->resident) {
            if (done) *done = 0;
            out->num_fluid = e->n;
            out->num_boundary = e->nb;
            return SPH_OK;
        }
        PoolScene t;
        SPH_CUDA(cudaMemcpyAsync(&t, table_.p + slot_of(id), sizeof t, cudaMemcpyDeviceToHost, st_));
        SPH_CUDA(cudaStreamSynchronize(st_));
        const DevScalars& s = t.s;
        out->time = s.time; out->dt = s.dt; out->avg_density_error = s.avgDensError;
        out->avg_divergence_error = s.avgDivError; out->max_velocity = s.maxVel; out->iterations = s.iterations;
        out->iterations_v = s.iterationsV; out->steps = s.steps; out->status = s.status;
#ifdef SPH_BOUNDS_CHECK
        // a bad index in any scene's list is reported with every scene
        unsigned faults = 0u;
        SPH_CUDA(cudaMemcpy(&faults, &pc_.p->faults, sizeof faults, cudaMemcpyDeviceToHost));
        out->status |= faults;
#endif
        out->sum_iterations = s.sumIterations; out->sum_iterations_v = s.sumIterationsV;
        out->num_fluid = t.n; out->num_boundary = t.nb;
        if (done) *done = t.running ? 0 : 1;
        return SPH_OK;
    }

    // Ids of resident scenes whose steps have completed (one table read).
    int poll(int* ids, int max, int* ndone)
    {
        if (S_) {
            k_pool_running<<<blocks(S_, 256), 256, 0, st_>>>(table_.p, S_, run_.p);
            SPH_CUDA(cudaGetLastError());
            SPH_CUDA(cudaMemcpyAsync(h_run_, run_.p, S_, cudaMemcpyDeviceToHost, st_));
        }
        SPH_CUDA(cudaStreamSynchronize(st_));
        int k = 0;
        for (uint32_t s = 0; s < S_; ++s)
            if (!h_run_[s] && !order_[s]->removed) {
                if (ids && k < max) ids[k] = order_[s]->id;
                ++k;
            }
        *ndone = k;
        return SPH_OK;
    }

    int download(int id, int field, double* out)
    {
        PoolEntry* e = find(id);
        if (!e || !e->resident) { fail("scene is not resident"); return SPH_ERR_INVALID; }
        // the layout fields of the scene's table entry, as the host keeps them
        const PoolScene& t = e->t;
        const bool bnd = field == SPH_FIELD_BOUNDARY_POSITION || field == SPH_FIELD_BOUNDARY_VOLUME;
        const uint32_t n = bnd ? t.nb : t.n, base = bnd ? t.bbase : t.pbase;
        const bool vec = field == SPH_FIELD_POSITION || field == SPH_FIELD_VELOCITY || field == SPH_FIELD_ACCELERATION ||
                         field == SPH_FIELD_BOUNDARY_POSITION;
        const P4<float>* v4 = nullptr;
        const float* sc = nullptr;
        int kind = 0;
        switch (field) {
            case SPH_FIELD_POSITION: v4 = pos_[cur_].p + base; kind = 1; break;
            case SPH_FIELD_VELOCITY: v4 = vel_[cur_].p + base; break;
            case SPH_FIELD_ACCELERATION: v4 = acc_.p + base; break;
            case SPH_FIELD_DENSITY: sc = rho_.p + base; kind = 2; break;
            case SPH_FIELD_ALPHA: sc = alpha_.p + base; kind = 2; break;
            case SPH_FIELD_PRED_DENSITY: sc = pred_[cur_].p + base; kind = 2; break;
            case SPH_FIELD_DIV_ERROR: sc = div_.p + base; kind = 2; break;
            case SPH_FIELD_KAPPA: sc = kappa_[cur_].p + base; kind = 2; break;
            case SPH_FIELD_KAPPA_V: sc = kappav_[cur_].p + base; kind = 2; break;
            case SPH_FIELD_BOUNDARY_POSITION: v4 = bpos_[bcur_].p + base; kind = 1; break;
            case SPH_FIELD_BOUNDARY_VOLUME: sc = bpsi_.p + base; kind = 2; break;
            default: fail("field not available in the pool"); return SPH_ERR_INVALID;
        }
        const size_t count = (size_t)n * (vec ? 3 : 1);
        if (!count) return SPH_OK;
        // a staging buffer kept between downloads (grow-only): no allocation,
        // and no cudaFree (which waits for the whole device) per call
        if (dl_.n < count) SPH_CUDA(dl_.alloc(std::max(count, dl_.n + dl_.n / 2)));
        const uint32_t* idp = bnd ? bid_[bcur_].p + base : id_[cur_].p + base;
        const uint32_t* cellp = bnd ? bcell_[bcur_].p + base : cell_[cur_].p + base;
        k_download<float><<<(n + 255) / 256, 256, 0, st_>>>(n, v4, sc, idp, cellp, t.g, (double)t.c.h, kind, dl_.p);
        SPH_CUDA(cudaGetLastError());
        SPH_CUDA(cudaMemcpyAsync(out, dl_.p, count * 8, cudaMemcpyDeviceToHost, st_));
        SPH_CUDA(cudaStreamSynchronize(st_));
        return SPH_OK;
    }

    // A resident scene's pair lists by scene-local original index (see
    // sph_pool_pair_lists).
    int pair_lists(int id, int* count, int* off, int* nbr, long long* total)
    {
        PoolEntry* e = find(id);
        if (!e || !e->resident) { fail("scene is not resident"); return SPH_ERR_INVALID; }
        const uint32_t s = slot_of(id);
        PoolScene t;
        SPH_CUDA(cudaMemcpyAsync(&t, table_.p + s, sizeof t, cudaMemcpyDeviceToHost, st_));
        SPH_CUDA(cudaStreamSynchronize(st_));
        const Lists<float> L = LS();
        const uint32_t* idp = id_[cur_].p;
        const uint32_t n = t.n, base = t.pbase, stride = N_;
        const cudaError_t err = dump_pair_lists(
            n, kmax_, st_,
            [&](const int* doff, int* dcnt, int* dn) {
                k_pair_lists<float><<<blocks(n, 256), 256, 0, st_>>>(n, base, stride, idp, L, doff, dcnt, dn);
            },
            count, off, nbr, total);
        SPH_CUDA(err);
        return SPH_OK;
    }

    int usage(unsigned long long* p, unsigned long long* b, unsigned long long* k, unsigned* s)
    {
        uint64_t P = 0, B = 0, K = 0;
        unsigned S = 0;
        for (auto& q : entries_) {
            if (q.removed) continue;
            P += q.n; B += q.nb; K += q.plan.nkeys; ++S;
        }
        if (p) *p = P;
        if (b) *b = B;
        if (k) *k = K;
        if (s) *s = S;
        return SPH_OK;
    }

    // Kernels of this library launched by steps so far.
    int launches(unsigned long long* out)
    {
        SPH_CUDA(cudaMemcpyAsync(h_pc_, pc_.p, sizeof(PoolCounters), cudaMemcpyDeviceToHost, st_));
        SPH_CUDA(cudaStreamSynchronize(st_));
        *out = host_launches_ + graph_launches_ + graph_period_kernels();
        return SPH_OK;
    }

private:
    PoolEntry* find(int id)
    {
        for (auto& e : entries_)
            if (e.id == id && !e.removed) return &e;
        return nullptr;
    }
    uint32_t slot_of(int id) const
    {
        for (uint32_t s = 0; s < S_; ++s)
            if (order_[s]->id == id) return s;
        return 0;
    }
    static unsigned blocks(size_t n, unsigned b) { return (unsigned)std::max<size_t>(1, (n + b - 1) / b); }

    Fluid<float> F(int k) const
    {
        Fluid<float> f{};
        f.pos = pos_[k].p; f.vel = vel_[k].p; f.kappa = kappa_[k].p; f.kappav = kappav_[k].p; f.pred = pred_[k].p;
        f.cell = cell_[k].p; f.id = id_[k].p;
        f.acc = acc_.p; f.xk = dummy4_.p; f.predR = dummy4_.p; f.predV = dummy4_.p; f.pacc = dummy4_.p;
        f.normal = normal_.p; f.rho = rho_.p; f.alpha = alpha_.p; f.div = div_.p; f.press = press_.p;
        f.n = N_;
        return f;
    }
    Boundary<float> B(int k) const { return Boundary<float>{bpos_[k].p, bpsi_.p, bcell_[k].p, bid_[k].p, NB_}; }
    Lists<float> LS() const
    {
        return Lists<float>{pairs_.p, lcount_.p, bgrad_.p, kbuf_.p, kmax_, posh_.p, &pc_.p->faults,
                            NB_ ? bposh_.p : nullptr, B(bcur_).cell};
    }

    int scan(uint32_t* out)
    {
        const unsigned per = (unsigned)tune_.scan_per;
        const unsigned nt = blocks(K_, kScanThreads * per);
        run("k_scan_tiles", [&] {
            if (per == 4) k_scan_tiles<4><<<nt, kScanThreads, 0, ls_>>>(K_, count_.p, out, tile_sums_.p);
            else if (per == 16) k_scan_tiles<16><<<nt, kScanThreads, 0, ls_>>>(K_, count_.p, out, tile_sums_.p);
            else k_scan_tiles<8><<<nt, kScanThreads, 0, ls_>>>(K_, count_.p, out, tile_sums_.p);
        });
        run("k_scan_tile_sums", [&] { k_scan_tile_sums<<<1, 1024, 0, ls_>>>(nt, tile_sums_.p, out, K_); });
        run("k_scan_add", [&] {
            if (per == 4) k_scan_add<4><<<nt, kScanThreads, 0, ls_>>>(K_, tile_sums_.p, out);
            else if (per == 16) k_scan_add<16><<<nt, kScanThreads, 0, ls_>>>(K_, tile_sums_.p, out);
            else k_scan_add<8><<<nt, kScanThreads, 0, ls_>>>(K_, tile_sums_.p, out);
        });
        SPH_CUDA(cudaGetLastError());
        return SPH_OK;
    }

    // ---- tuned launches ---------------------------------------------------
    // Shapes: (threads per block, threads per SM the register budget allows).
    // DIV0: the build also forms the divergence solve's first error pass.
    template <bool DIV0 = false> void launch_build(Fluid<float> f, const P4<float>* bp, Lists<float> L)
    {
        const int bb = tune_.build_block, bo = tune_.build_occ;
        const uint32_t qd = (uint32_t)tune_.queue;
        const size_t smem = (size_t)qd * (size_t)bb * sizeof(uint32_t);
#define SPH_BUILD(BL, MB) \
    k_pool_build_lists<BL, MB, DIV0><<<blocks(N_, BL), BL, smem, ls_>>>(f, bp, sid_.p, table_.p, starts_.p, bstarts_.p, L, qd)
        if (bb == 128 && bo == 896) SPH_BUILD(128, 7);
        else if (bb == 128) SPH_BUILD(128, 8);
        else if (bo == 1024) SPH_BUILD(256, 4);
        else SPH_BUILD(256, 3);
#undef SPH_BUILD
    }
    template <int MODE> void launch_correct(Fluid<float> f, const P4<float>* bp, Lists<float> L)
    {
        const int sb = tune_.solver_block, so = tune_.solver_occ;
#define SPH_CORR(BL, MB) \
    k_pool_correct<BL, MB, MODE><<<blocks(N_, BL), BL, 0, ls_>>>(f, bp, sid_.p, table_.p, starts_.p, bstarts_.p, L)
        if (sb == 128) { if (so == 1536) SPH_CORR(128, 12); else if (so == 2048) SPH_CORR(128, 16); else SPH_CORR(128, 8); }
        else { if (so == 1536) SPH_CORR(256, 6); else if (so == 2048) SPH_CORR(256, 8); else SPH_CORR(256, 4); }
#undef SPH_CORR
    }
    template <bool DIV, bool INITIAL> void launch_errors(Fluid<float> f, const P4<float>* bp, Lists<float> L)
    {
        const int sb = tune_.solver_block, so = tune_.solver_occ;
#define SPH_ERRS(BL, MB) \
    k_pool_errors<BL, MB, DIV, INITIAL><<<blocks(N_, BL), BL, 0, ls_>>>(f, bp, sid_.p, table_.p, starts_.p, bstarts_.p, L)
        if (sb == 128) { if (so == 1536) SPH_ERRS(128, 12); else if (so == 2048) SPH_ERRS(128, 16); else SPH_ERRS(128, 8); }
        else { if (so == 1536) SPH_ERRS(256, 6); else if (so == 2048) SPH_ERRS(256, 8); else SPH_ERRS(256, 4); }
#undef SPH_ERRS
    }

    // Launch accounting: kernels of host-driven steps are counted as they
    // are launched, those of a captured step graph per loop part.
    template <typename Fn> void run(const char* name, Fn&& fn)
    {
        if (capturing_) { ++cap_[loop_ctx_]; fn(); return; }
        if (counting_) ++host_launches_;
        int fam = -1, sub = 0;
        if (tuning_) tune_family(name, &fam, &sub);
        const bool prof = prof_ && counting_;
        if (fam < 0 && !prof) { fn(); return; }
        cudaEvent_t a = take_event(), b = take_event();
        cudaEvent_t c = prof && fam >= 0 ? take_event() : nullptr, d = c ? take_event() : nullptr;
        cudaEventRecord(a, ls_);
        if (c) cudaEventRecord(c, ls_);
        fn();
        if (d) cudaEventRecord(d, ls_);
        cudaEventRecord(b, ls_);
        if (fam >= 0) tpending_.push_back({fam, sub, a, b});
        else pending_.push_back({name, a, b});
        if (c) pending_.push_back({name, c, d});
    }
    cudaEvent_t take_event()
    {
        if (!events_.empty()) { cudaEvent_t e = events_.back(); events_.pop_back(); return e; }
        cudaEvent_t e;
        cudaEventCreate(&e);
        return e;
    }
    DevScalars* scalars_of(uint32_t s) const
    {
        return reinterpret_cast<DevScalars*>(reinterpret_cast<char*>(table_.p + s) + offsetof(PoolScene, s));
    }

    // Applies admissions and removals: repack, upload, sort, lists.
    int relayout()
    {
        SPH_CUDA(cudaStreamSynchronize(st_));
        graph_period_end();
        counting_ = false;
        // device-side scene state of the resident scenes back to the host
        if (S_) {
            std::vector<PoolScene> t(S_);
            SPH_CUDA(cudaMemcpy(t.data(), table_.p, S_ * sizeof(PoolScene), cudaMemcpyDeviceToHost));
            for (uint32_t s = 0; s < S_; ++s) order_[s]->t = t[s];
        }
        std::vector<PoolEntry*> keep, fresh;
        for (auto& e : entries_) {
            if (e.removed) continue;
            (e.resident ? keep : fresh).push_back(&e);
        }
        std::vector<PoolEntry*> order = keep;
        order.insert(order.end(), fresh.begin(), fresh.end());
        // layout: packed in order
        std::vector<uint32_t> pb(order.size()), bb(order.size()), kb(order.size()), mxo(order.size()), myo(order.size());
        uint64_t P = 0, Bn = 0, K = 0, MX = 0;
        for (size_t s = 0; s < order.size(); ++s) {
            pb[s] = (uint32_t)P; bb[s] = (uint32_t)Bn; kb[s] = (uint32_t)K;
            mxo[s] = (uint32_t)MX; MX += order[s]->plan.nn[0];
            myo[s] = (uint32_t)MX; MX += order[s]->plan.nn[1];
            P += order[s]->n; Bn += order[s]->nb; K += order[s]->plan.nkeys;
        }
        // morton tables of every resident scene
        std::vector<uint32_t> mort(std::max<uint64_t>(MX, 1));
        for (size_t s = 0; s < order.size(); ++s) {
            std::copy(order[s]->plan.mx.begin(), order[s]->plan.mx.end(), mort.begin() + mxo[s]);
            std::copy(order[s]->plan.my.begin(), order[s]->plan.my.end(), mort.begin() + myo[s]);
        }
        SPH_CUDA(mort_.alloc(mort.size()));
        SPH_CUDA(cudaMemcpyAsync(mort_.p, mort.data(), mort.size() * 4, cudaMemcpyHostToDevice, st_));
        const int nc = 1 - cur_, nbc = 1 - bcur_;
        // repack kept scenes into the other buffers
        if (!keep.empty()) {
            std::vector<uint32_t> a(keep.size()), b(keep.size()), l(keep.size()), ba(keep.size()), bbb(keep.size()),
                bl(keep.size());
            for (size_t s = 0; s < keep.size(); ++s) {
                a[s] = pb[s]; b[s] = keep[s]->t.pbase; l[s] = keep[s]->n;
                ba[s] = bb[s]; bbb[s] = keep[s]->t.bbase; bl[s] = keep[s]->nb;
            }
            const uint32_t Sk = (uint32_t)keep.size();
            uint32_t Pk = 0, Bk = 0;
            for (auto* e : keep) { Pk += e->n; Bk += e->nb; }
            SPH_CUDA(cudaMemcpyAsync(seg_a_.p, a.data(), Sk * 4, cudaMemcpyHostToDevice, st_));
            SPH_CUDA(cudaMemcpyAsync(seg_b_.p, b.data(), Sk * 4, cudaMemcpyHostToDevice, st_));
            SPH_CUDA(cudaMemcpyAsync(seg_n_.p, l.data(), Sk * 4, cudaMemcpyHostToDevice, st_));
            k_repack_fluid<<<blocks(Pk, 256), 256, 0, st_>>>(Pk, seg_a_.p, seg_b_.p, seg_n_.p, Sk, F(cur_), F(nc));
            SPH_CUDA(cudaGetLastError());
            SPH_CUDA(cudaStreamSynchronize(st_));
            if (Bk) {
                SPH_CUDA(cudaMemcpyAsync(seg_a_.p, ba.data(), Sk * 4, cudaMemcpyHostToDevice, st_));
                SPH_CUDA(cudaMemcpyAsync(seg_b_.p, bbb.data(), Sk * 4, cudaMemcpyHostToDevice, st_));
                SPH_CUDA(cudaMemcpyAsync(seg_n_.p, bl.data(), Sk * 4, cudaMemcpyHostToDevice, st_));
                k_repack_boundary<<<blocks(Bk, 256), 256, 0, st_>>>(Bk, seg_a_.p, seg_b_.p, seg_n_.p, Sk, B(bcur_), B(nbc));
                SPH_CUDA(cudaGetLastError());
                SPH_CUDA(cudaStreamSynchronize(st_));
            }
        }
        N_ = (uint32_t)P;
        NB_ = (uint32_t)Bn;
        K_ = (uint32_t)K;
        // scene table
        std::vector<PoolScene> tab(order.size());
        for (size_t s = 0; s < order.size(); ++s) {
            PoolEntry* e = order[s];
            PoolScene t = e->t;
            if (!e->resident && e->restored) {
                t.s = e->snap_s;
                t.s.block_counter = 0;
                t.acc = 0;
                t.steps_left = e->steps;
                t.running = e->steps > 0;
                t.loop_active = 0;
                t.vmax_bits = 0;
                t.bad = 0;
                t.akinci = 1;
            } else if (!e->resident) {
                t.s = DevScalars{};
                t.s.dt = e->d.time_step;
                t.acc = 0;
                t.steps_left = e->steps;
                t.running = e->steps > 0;
                t.loop_active = 0;
                t.vmax_bits = 0;
                t.bad = 0;
                t.akinci = 1;
            }
            t.g.nx = e->plan.nn[0]; t.g.ny = e->plan.nn[1]; t.g.nz = e->plan.nn[2];
            t.g.ox = e->plan.o[0]; t.g.oy = e->plan.o[1]; t.g.oz = e->plan.o[2];
            t.g.mortx = mort_.p + mxo[s];
            t.g.morty = mort_.p + myo[s];
            t.key_base = kb[s]; t.n = e->n; t.nb = e->nb; t.pbase = pb[s]; t.bbase = bb[s];
            t.eclamp = (float)(kErrBudget / (double)std::max(e->n, 1u));
            tab[s] = t;
        }
        S_ = (uint32_t)order.size();
        SPH_CUDA(cudaMemcpyAsync(table_.p, tab.data(), S_ * sizeof(PoolScene), cudaMemcpyHostToDevice, st_));
        // upload the new scenes into their segments from their staged points
        // (one wait for all of them); the arena is then free again
        for (size_t s = keep.size(); s < order.size(); ++s) {
            PoolEntry* e = order[s];
            if (e->restored) {
                // the snapshot's arrays as they were stored
                size_t L[11];
                snap_layout(e->n, e->nb, L);
                const char* a = reinterpret_cast<const char*>(arena_.p + e->ox);
                const size_t n = e->n, nb = e->nb;
                void* dst[10] = {pos_[nc].p + pb[s], vel_[nc].p + pb[s], kappa_[nc].p + pb[s], kappav_[nc].p + pb[s],
                                 pred_[nc].p + pb[s], cell_[nc].p + pb[s], id_[nc].p + pb[s], bpos_[nbc].p + bb[s],
                                 bcell_[nbc].p + bb[s], bid_[nbc].p + bb[s]};
                const size_t sz[10] = {16 * n, 16 * n, 4 * n, 4 * n, 4 * n, 4 * n, 4 * n, 16 * nb, 4 * nb, 4 * nb};
                for (int k = 0; k < 10; ++k)
                    if (sz[k]) SPH_CUDA(cudaMemcpyAsync(dst[k], a + L[k], sz[k], cudaMemcpyDeviceToDevice, st_));
                SPH_CUDA(cudaMemsetAsync(acc_.p + pb[s], 0, n * sizeof(P4<float>), st_));
                SPH_CUDA(cudaMemsetAsync(press_.p + pb[s], 0, n * sizeof(float), st_));
                e->staged = false;
                e->restored = false;
                e->resident = true;
                continue;
            }
            Fluid<float> f = F(nc);
            f.pos += pb[s]; f.vel += pb[s]; f.kappa += pb[s]; f.kappav += pb[s]; f.cell += pb[s]; f.id += pb[s];
            f.acc += pb[s]; f.press += pb[s];
            DevScalars* sst = scalars_of(s);
            k_upload_fluid<float><<<blocks(e->n, 256), 256, 0, st_>>>(arena_.p + e->ox, arena_.p + e->ov, e->n, 0, f,
                                                                      tab[s].g, 4.0 * e->d.particle_radius, sst);
            SPH_CUDA(cudaMemsetAsync(pred_[nc].p + pb[s], 0, e->n * sizeof(float), st_));
            if (e->nb) {
                Boundary<float> bo = B(nbc);
                bo.pos += bb[s]; bo.cell += bb[s]; bo.id += bb[s];
                k_upload_boundary<float><<<blocks(e->nb, 256), 256, 0, st_>>>(arena_.p + e->ob, e->nb, bo, tab[s].g,
                                                                              4.0 * e->d.particle_radius, sst);
            }
            SPH_CUDA(cudaGetLastError());
            e->staged = false;
            e->resident = true;
        }
        SPH_CUDA(cudaStreamSynchronize(st_));
        arena_used_ = 0;
        cur_ = nc;
        bcur_ = nbc;
        // drop removed entries; the resident order is the layout order
        entries_.remove_if([](const PoolEntry& e) { return e.removed; });
        order_ = order;
        any_forces_ = any_st_ = false;
        for (uint32_t s = 0; s < S_; ++s) {
            order_[s]->t = tab[s];
            any_forces_ |= (tab[s].c.force_flags & kPoolForces) != 0;
            any_st_ |= (tab[s].c.force_flags & F_SURFACE_TENSION) != 0;
        }
        // scene ids of fluid and boundary particles
        std::vector<uint32_t> pbv(pb.begin(), pb.end()), bbv(bb.begin(), bb.end());
        SPH_CUDA(cudaMemcpyAsync(seg_a_.p, pbv.data(), S_ * 4, cudaMemcpyHostToDevice, st_));
        k_fill_sid<<<blocks(N_, 256), 256, 0, st_>>>(N_, seg_a_.p, S_, sid_.p);
        SPH_CUDA(cudaStreamSynchronize(st_));
        if (NB_) {
            SPH_CUDA(cudaMemcpyAsync(seg_a_.p, bbv.data(), S_ * 4, cudaMemcpyHostToDevice, st_));
            k_fill_sid<<<blocks(NB_, 256), 256, 0, st_>>>(NB_, seg_a_.p, S_, bsid_.p);
            SPH_CUDA(cudaStreamSynchronize(st_));
        }
        // boundary: sort by (key, id) -- kept scenes are already in order -- and volumes
        if (NB_) {
            k_pool_bcount<<<blocks(NB_, 256), 256, 0, st_>>>(NB_, B(bcur_), bsid_.p, table_.p, key_.p, slot_.p, count_.p);
            int rc = scan(bstarts_.p);
            if (rc) return rc;
            k_scatter<<<blocks(NB_, 256), 256, 0, st_>>>(NB_, key_.p, slot_.p, bstarts_.p, tmp_.p);
            k_gather_boundary<float><<<blocks(NB_, 256), 256, 0, st_>>>(NB_, tmp_.p, key_.p, bstarts_.p, B(bcur_), B(1 - bcur_));
            SPH_CUDA(cudaGetLastError());
            bcur_ = 1 - bcur_;
            k_pool_psi<<<blocks(NB_, 128), 128, 0, st_>>>(NB_, B(bcur_), bsid_.p, table_.p, bstarts_.p);
            SPH_CUDA(cudaGetLastError());
            k_pool_boundary_half<<<blocks(NB_, 256), 256, 0, st_>>>(NB_, B(bcur_), bsid_.p, table_.p, bposh_.p);
            SPH_CUDA(cudaGetLastError());
        } else {
            SPH_CUDA(cudaMemsetAsync(bstarts_.p, 0, (K_ + 1) * sizeof(uint32_t), st_));
        }
        // fluid grid and lists (DFSPHSolver::init for new scenes; identical
        // recomputation for the kept ones, whose positions have not moved)
        int rc = build_grid(false);
        if (rc) return rc;
        run("k_pool_build_lists", [&] { launch_build(F(cur_), bpos_[bcur_].p, LS()); });
        SPH_CUDA(cudaGetLastError());
        SPH_CUDA(cudaStreamSynchronize(st_));
        counting_ = true;
        drop_graphs();
        dirty_ = false;
        graph_period_begin();
        tune_after_relayout();
        return SPH_OK;
    }

    int build_grid(bool move)
    {
        Fluid<float> a = F(cur_);
        if (move)
            run("k_pool_cell_update", [&] { k_pool_cell_update<true><<<blocks(N_, 256), 256, 0, ls_>>>(N_, a, sid_.p, table_.p, key_.p, slot_.p, count_.p); });
        else
            run("k_pool_cell_update", [&] { k_pool_cell_update<false><<<blocks(N_, 256), 256, 0, ls_>>>(N_, a, sid_.p, table_.p, key_.p, slot_.p, count_.p); });
        SPH_CUDA(cudaGetLastError());
        int rc = scan(starts_.p);
        if (rc) return rc;
        run("k_scatter", [&] { k_scatter<<<blocks(N_, 256), 256, 0, ls_>>>(N_, key_.p, slot_.p, starts_.p, tmp_.p); });
        run("k_gather_fluid", [&] { k_gather_fluid<float><<<blocks(N_, 256), 256, 0, ls_>>>(N_, tmp_.p, key_.p, starts_.p, F(cur_), F(1 - cur_),
                                                                                          posh_.p); });
        SPH_CUDA(cudaGetLastError());
        cur_ = 1 - cur_;
        return SPH_OK;
    }

    template <typename Init, typename Body> int solve_loop(int loop_id, Init&& init, Body&& body)
    {
        if (capturing_) {
            cudaStreamCaptureStatus cs;
            cudaGraph_t g;
            const cudaGraphNode_t* deps = nullptr;
            size_t ndeps = 0;
            SPH_CUDA(cudaStreamGetCaptureInfo(st_, &cs, nullptr, &g, nullptr, nullptr, nullptr));
            cudaGraphConditionalHandle h;
            SPH_CUDA(cudaGraphConditionalHandleCreate(&h, g, 0, 0));
            init(h);
            SPH_CUDA(cudaGetLastError());
            SPH_CUDA(cudaStreamGetCaptureInfo(st_, &cs, nullptr, &g, &deps, nullptr, &ndeps));
            cudaGraphNodeParams p{};
            p.type = cudaGraphNodeTypeConditional;
            p.conditional.handle = h;
            p.conditional.type = cudaGraphCondTypeWhile;
            p.conditional.size = 1;
            cudaGraphNode_t node;
            SPH_CUDA(cudaGraphAddNode(&node, g, deps, nullptr, ndeps, &p));
            cudaGraph_t bodyg = p.conditional.phGraph_out[0];
            SPH_CUDA(cudaStreamUpdateCaptureDependencies(st_, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
            SPH_CUDA(cudaStreamBeginCaptureToGraph(st2_, bodyg, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
            ls_ = st2_;
            loop_ctx_ = loop_id;
            body(h);
            loop_ctx_ = 0;
            ls_ = st_;
            cudaGraph_t out;
            SPH_CUDA(cudaStreamEndCapture(st2_, &out));
            return SPH_OK;
        }
        init((cudaGraphConditionalHandle)0);
        SPH_CUDA(cudaGetLastError());
        for (unsigned it = 0; it < 1000u; ++it) {
            SPH_CUDA(cudaMemcpyAsync(h_pc_, pc_.p, sizeof(PoolCounters), cudaMemcpyDeviceToHost, st_));
            SPH_CUDA(cudaStreamSynchronize(st_));
            if (!h_pc_->any) break;
            if (loop_id == 1) ++host_body_d_; else ++host_body_v_;
            body((cudaGraphConditionalHandle)0);
            SPH_CUDA(cudaGetLastError());
        }
        return SPH_OK;
    }

    // DFSPHSolver::step (DFSPHSolver.cpp:38-112) for every running scene.
    int one_step()
    {
        const unsigned nb = blocks(N_, kBlock);
        const unsigned nb256 = blocks(N_, 256);
        {
            Fluid<float> f = F(cur_);
            const P4<float>* bp = bpos_[bcur_].p;
            Lists<float> L = LS();
            if (any_st_ || any_forces_) {
                auto ph = phase("npForces");
                if (any_st_)
                    run("k_pool_st_normals", [&] { k_pool_st_normals<<<nb, kBlock, 0, ls_>>>(f, sid_.p, table_.p, starts_.p); });
                if (any_forces_)
                    run("k_pool_npforce", [&] { k_pool_npforce<<<nb, kBlock, 0, ls_>>>(f, bp, sid_.p, table_.p, starts_.p, bstarts_.p); });
            }
            run("k_pool_cfl_accum", [&] { k_pool_cfl_accum<<<nb256, 256, 0, ls_>>>(f, sid_.p, table_.p); });
            run("k_pool_cfl_control", [&] { k_pool_cfl_control<<<1, 256, 0, ls_>>>(table_.p, S_); });
            run("k_pool_predict_v_warm", [&] { k_pool_predict_v_warm<<<nb256, 256, 0, ls_>>>(f, sid_.p, table_.p, L.kbuf); });
            auto ph = phase("Density solver");
            run("k_pool_correct", [&] { launch_correct<0>(f, bp, L); });
            SPH_CUDA(cudaGetLastError());
            int rc = solve_loop(
                1,
                [&](cudaGraphConditionalHandle h) {
                    run("k_pool_errors_density", [&] { launch_errors<false, true>(f, bp, L); });
                    run("k_pool_control", [&] { k_pool_control<0><<<1, 256, 0, ls_>>>(table_.p, S_, pc_.p, h); });
                },
                [&](cudaGraphConditionalHandle h) {
                    run("k_pool_correct", [&] { launch_correct<1>(f, bp, L); });
                    run("k_pool_errors_density", [&] { launch_errors<false, false>(f, bp, L); });
                    run("k_pool_control", [&] { k_pool_control<1><<<1, 256, 0, ls_>>>(table_.p, S_, pc_.p, h); });
                });
            if (rc) return rc;
        }
        int rc;
        {
            auto ph = phase("Fill grid");  // with the position update fused in
            rc = build_grid(true);
        }
        if (rc) return rc;
        {
            Fluid<float> f = F(cur_);
            const P4<float>* bp = bpos_[bcur_].p;
            Lists<float> L = LS();
            // the build also forms the divergence solve's first error pass
            {
                auto ph = phase("Neigh search+Densities+Alpha factor");
                run("k_pool_build_lists", [&] { launch_build<true>(f, bp, L); });
            }
            SPH_CUDA(cudaGetLastError());
            auto ph = phase("Divergence solver");
            rc = solve_loop(
                2,
                [&](cudaGraphConditionalHandle h) {
                    run("k_pool_control", [&] { k_pool_control<2><<<1, 256, 0, ls_>>>(table_.p, S_, pc_.p, h); });
                },
                [&](cudaGraphConditionalHandle h) {
                    run("k_pool_correct", [&] { launch_correct<2>(f, bp, L); });
                    run("k_pool_errors_div", [&] { launch_errors<true, false>(f, bp, L); });
                    run("k_pool_control", [&] { k_pool_control<3><<<1, 256, 0, ls_>>>(table_.p, S_, pc_.p, h); });
                });
            if (rc) return rc;
        }
        run("k_pool_finish", [&] { k_pool_finish<<<1, 256, 0, ls_>>>(table_.p, S_); });
        SPH_CUDA(cudaGetLastError());
        return SPH_OK;
    }

    int graph_step()
    {
        const int k = cur_;
        if (!gexec_[k]) {
            cudaGraph_t g;
            SPH_CUDA(cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal));
            capturing_ = true;
            cap_[0] = cap_[1] = cap_[2] = 0;
            const int rc = one_step();
            capturing_ = false;
            cudaError_t e = cudaStreamEndCapture(st_, &g);
            if (rc) { if (e == cudaSuccess) cudaGraphDestroy(g); cur_ = k; return rc; }
            SPH_CUDA(e);
            SPH_CUDA(cudaGraphInstantiate(&gexec_[k], g, 0));
            cudaGraphDestroy(g);
            cur_ = k;
            // the loop-control kernel is part of each body and of the fixed part
            fixed_ = cap_[0];
            body_d_size_ = cap_[1];
            body_v_size_ = cap_[2];
        }
        SPH_CUDA(cudaGraphLaunch(gexec_[k], st_));
        ++gsteps_;
        cur_ = 1 - k;
        return SPH_OK;
    }

    // Graph kernels of the current layout (h_pc_ must be current).  Loop
    // bodies are counted from the device's body counters, which host-driven
    // steps advance too; those are subtracted via host_body_*.
    unsigned long long graph_period_kernels() const
    {
        if (!gsteps_) return 0ull;
        return gsteps_ * fixed_ + body_d_size_ * (h_pc_->body_d - snap_d_ - host_body_d_) +
               body_v_size_ * (h_pc_->body_v - snap_v_ - host_body_v_);
    }
    void graph_period_begin()
    {
        cudaMemcpy(h_pc_, pc_.p, sizeof(PoolCounters), cudaMemcpyDeviceToHost);
        snap_d_ = h_pc_->body_d;
        snap_v_ = h_pc_->body_v;
        host_body_d_ = host_body_v_ = 0;
        gsteps_ = 0;
    }
    void graph_period_end()
    {
        cudaMemcpy(h_pc_, pc_.p, sizeof(PoolCounters), cudaMemcpyDeviceToHost);
        graph_launches_ += graph_period_kernels();
    }

public:
    unsigned long long total_launches()
    {
        unsigned long long k = 0;
        launches(&k);
        return k;
    }

private:
    sph_pool_desc pd_{};
    cudaStream_t st_ = nullptr, st2_ = nullptr, ls_ = nullptr;
    PoolCounters* h_pc_ = nullptr;
    std::list<PoolEntry> entries_;  // stable addresses: order_ points into it
    std::vector<PoolEntry*> order_;
    int next_id_ = 1;
    bool dirty_ = false, graph_ = false, capturing_ = false;
    uint32_t S_ = 0, N_ = 0, NB_ = 0, K_ = 0, kmax_ = 64;
    int cur_ = 0, bcur_ = 0;
    int loop_ctx_ = 0;
    unsigned cap_[3] = {0, 0, 0};
    unsigned long long fixed_ = 0, body_d_size_ = 0, body_v_size_ = 0, gsteps_ = 0, snap_d_ = 0, snap_v_ = 0;
    unsigned long long host_launches_ = 0, graph_launches_ = 0, host_body_d_ = 0, host_body_v_ = 0;
    bool counting_ = true, any_forces_ = false, any_st_ = false, prof_ = false, tuning_ = false;
    PhaseLog phases_;
    Tune tune_;
    int tune_mode_ = 1, tune_source_ = 0, tune_left_ = 0, tune_step_ = 0;
    unsigned long long tune_bucket_ = 0;
    int cand_[3] = {0, 0, 0};
    double tacc_ms_[3][12][3];
    unsigned tacc_n_[3][12][3];
    std::string tune_log_;
    struct TTimed { int fam, sub; cudaEvent_t a, b; };
    std::vector<TTimed> tpending_;
    struct Timed { const char* name; cudaEvent_t a, b; };
    std::vector<Timed> pending_;
    std::vector<cudaEvent_t> events_;
    cudaEvent_t tev_[2] = {nullptr, nullptr};
    cudaGraphExec_t gexec_[2] = {nullptr, nullptr};
    DevBuf<P4<float>> pos_[2], vel_[2], bpos_[2];
    DevBuf<float> kappa_[2], kappav_[2], pred_[2];
    DevBuf<uint32_t> cell_[2], id_[2], bcell_[2], bid_[2];
    DevBuf<P4<float>> acc_, dummy4_, pairs_, bgrad_, normal_;
    DevBuf<uint4> posh_;  // half-precision positions for the build's cull (particle pairs)
    DevBuf<uint4> bposh_; // the boundary points' half-precision copy (boundary cull)
    DevBuf<uint8_t> run_;   // per scene: running (poll)
    uint8_t* h_run_ = nullptr;
    DevBuf<float> rho_, alpha_, div_, press_, kbuf_, bpsi_;
    DevBuf<uint32_t> sid_, bsid_, lcount_, key_, slot_, tmp_, count_, starts_, bstarts_, tile_sums_, mort_;
    DevBuf<uint32_t> seg_a_, seg_b_, seg_n_;
    DevBuf<PoolScene> table_;
    DevBuf<PoolCounters> pc_;
    cudaStream_t up_ = nullptr;   // admissions: the new scenes' points to the device
    DevBuf<double> arena_;        // their staging (grow-only; emptied by each re-layout)
    size_t arena_used_ = 0;
    DevBuf<double> box_;          // admissions: per-block bounding boxes of the staged points
    double* h_box_ = nullptr;
    DevBuf<double> dl_;           // downloads: original-order FP64 staging (grow-only)
};

}  // namespace sph

// Calls on one pool are serialised (a submitting thread and a stepping
// thread may share it) and run on the device the pool was created on.
struct sph_pool {
    sph::Pool pool;
    std::mutex m;
    int device = 0;
};

namespace {
struct PoolLock {
    std::lock_guard<std::mutex> lk;
    explicit PoolLock(sph_pool* p) : lk(p->m) { cudaSetDevice(p->device); }
};
}  // namespace

static int pool_bad(sph_pool* p, const char* m)
{
    if (p) p->pool.err = m;
    return SPH_ERR_INVALID;
}

extern "C" {

int sph_pool_desc_from_budget(unsigned long long hbm_bytes, int neighbor_list_max, sph_pool_desc* out)
{
    if (!out || hbm_bytes < (1ull << 20)) return SPH_ERR_INVALID;
    const unsigned long long kmax = neighbor_list_max > 0 ? (unsigned long long)neighbor_list_max : 64ull;
    // bytes per fluid particle (double-buffered carried state, shared fields
    // with the half-precision positions and the surface normals, sort
    // scratch, pair-list slots), per boundary particle and per grid key, with
    // one boundary particle and sixteen keys budgeted per fluid particle
    const unsigned long long per_p = 2 * (16 + 16 + 4 + 4 + 4 + 4 + 4) +
                                     (16 + 4 + 4 + 4 + 4 + 4 + 4 + 4 + 16 + 8 + 16) + 3 * 4 + kmax * 16;
    const unsigned long long per_b = 2 * (16 + 4 + 4) + 4 + 4;
    const unsigned long long per_k = 3 * 4;
    const unsigned long long unit = per_p + per_b + 16 * per_k;
    std::memset(out, 0, sizeof *out);
    out->max_particles = hbm_bytes / unit;
    out->max_boundary = out->max_particles;
    out->max_keys = 16 * out->max_particles;
    out->max_scenes = 4096;
    out->neighbor_list_max = (int)kmax;
    if (out->max_particles >= (1ull << 31)) {
        out->max_particles = (1ull << 31) - 1;
        out->max_boundary = out->max_particles;
        out->max_keys = (1ull << 31) - 1;
    }
    return SPH_OK;
}

int sph_pool_create(const sph_pool_desc* desc, sph_pool** out)
{
    if (!desc || !out) return SPH_ERR_INVALID;
    *out = nullptr;
    sph_pool* p = new (std::nothrow) sph_pool();
    if (!p) return SPH_ERR_INVALID;
    cudaGetDevice(&p->device);
    const int rc = p->pool.create(*desc);
    if (rc) {
        delete p;
        return rc;
    }
    *out = p;
    return SPH_OK;
}

int sph_pool_destroy(sph_pool* p)
{
    if (!p) return SPH_ERR_INVALID;
    delete p;
    return SPH_OK;
}

int sph_pool_add_scene(sph_pool* p, const sph_scene_desc* d, const double* x, const double* v, unsigned n,
                       const double* bx, unsigned nb, unsigned steps, int* scene_id)
{
    if (!p || !d || !scene_id || (nb && !bx)) return pool_bad(p, "invalid argument");
    PoolLock lock(p);
    return p->pool.add(*d, x, v, n, bx, nb, steps, scene_id);
}

int sph_pool_remove_scene(sph_pool* p, int scene_id)
{
    if (!p) return SPH_ERR_INVALID;
    PoolLock lock(p);
    return p->pool.remove(scene_id);
}

int sph_pool_step(sph_pool* p, int nsteps)
{
    if (!p || nsteps < 0) return pool_bad(p, "invalid argument");
    PoolLock lock(p);
    return p->pool.step(nsteps);
}

int sph_pool_set_graph(sph_pool* p, int enable)
{
    if (!p) return SPH_ERR_INVALID;
    PoolLock lock(p);
    return p->pool.set_graph(enable);
}

int sph_pool_synchronize(sph_pool* p)
{
    if (!p) return SPH_ERR_INVALID;
    PoolLock lock(p);
    return p->pool.sync();
}

int sph_pool_query(sph_pool* p, int scene_id, sph_stats* out, int* done)
{
    if (!p || !out) return pool_bad(p, "invalid argument");
    PoolLock lock(p);
    return p->pool.query(scene_id, out, done);
}

int sph_pool_poll(sph_pool* p, int* done_ids, int max_ids, int* num_done)
{
    if (!p || !num_done) return pool_bad(p, "invalid argument");
    PoolLock lock(p);
    return p->pool.poll(done_ids, max_ids, num_done);
}

int sph_pool_download(sph_pool* p, int scene_id, int field, double* out)
{
    if (!p || !out) return pool_bad(p, "invalid argument");
    PoolLock lock(p);
    return p->pool.download(scene_id, field, out);
}

int sph_pool_pair_lists(sph_pool* p, int scene_id, int* count, int* off, int* nbr, long long* total)
{
    if (!p || (nbr && !off)) return pool_bad(p, "invalid argument");
    PoolLock lock(p);
    return p->pool.pair_lists(scene_id, count, off, nbr, total);
}

int sph_pool_snapshot(sph_pool* p, int scene_id, void* buf, unsigned long long capacity, unsigned long long* size)
{
    if (!p || !size) return pool_bad(p, "invalid argument");
    PoolLock lock(p);
    return p->pool.snapshot(scene_id, buf, capacity, size);
}

int sph_pool_restore(sph_pool* p, const void* buf, unsigned long long size, unsigned steps, int* scene_id)
{
    if (!p || !buf || !scene_id) return pool_bad(p, "invalid argument");
    PoolLock lock(p);
    return p->pool.restore(buf, size, steps, scene_id);
}

int sph_pool_usage(sph_pool* p, unsigned long long* particles, unsigned long long* boundary, unsigned long long* keys,
                   unsigned* scenes)
{
    if (!p) return SPH_ERR_INVALID;
    PoolLock lock(p);
    return p->pool.usage(particles, boundary, keys, scenes);
}

int sph_pool_get_launch_count(sph_pool* p, unsigned long long* out)
{
    if (!p || !out) return pool_bad(p, "invalid argument");
    PoolLock lock(p);
    *out = p->pool.total_launches();
    return SPH_OK;
}

int sph_pool_step_timed(sph_pool* p, int nsteps, float* elapsed_ms)
{
    if (!p || nsteps < 0 || !elapsed_ms) return pool_bad(p, "invalid argument");
    PoolLock lock(p);
    return p->pool.step_timed(nsteps, elapsed_ms);
}

int sph_pool_set_profiling(sph_pool* p, int enable)
{
    if (!p) return SPH_ERR_INVALID;
    PoolLock lock(p);
    return p->pool.set_profiling(enable);
}

int sph_pool_get_profile(sph_pool* p, char* buf, unsigned long long len)
{
    if (!p) return SPH_ERR_INVALID;
    PoolLock lock(p);
    return p->pool.profile(buf, (size_t)len);
}

int sph_pool_get_phase_profile(sph_pool* p, char* buf, unsigned long long len)
{
    if (!p) return SPH_ERR_INVALID;
    PoolLock lock(p);
    return p->pool.phase_profile(buf, (size_t)len);
}

int sph_pool_set_autotune(sph_pool* p, int mode)
{
    if (!p) return SPH_ERR_INVALID;
    PoolLock lock(p);
    return p->pool.set_autotune(mode);
}

int sph_pool_get_tuning(sph_pool* p, sph_pool_tuning* out)
{
    if (!p || !out) return pool_bad(p, "invalid argument");
    PoolLock lock(p);
    p->pool.get_tuning(out);
    return SPH_OK;
}

int sph_pool_set_tuning(sph_pool* p, const sph_pool_tuning* t)
{
    if (!p || !t) return pool_bad(p, "invalid argument");
    PoolLock lock(p);
    return p->pool.set_tuning(*t);
}

int sph_pool_get_tuning_log(sph_pool* p, char* buf, unsigned long long len)
{
    if (!p) return SPH_ERR_INVALID;
    PoolLock lock(p);
    const std::string& s = p->pool.tuning_log();
    if (buf && len) {
        std::strncpy(buf, s.c_str(), (size_t)len - 1);
        buf[len - 1] = 0;
    }
    return (int)s.size();
}

int sph_pool_list_pairs(sph_pool* p, unsigned long long* pairs, unsigned* overflow)
{
    if (!p || !pairs || !overflow) return pool_bad(p, "invalid argument");
    PoolLock lock(p);
    return p->pool.list_pairs(pairs, overflow);
}

int sph_pool_count_work(sph_pool* p, unsigned long long* out)
{
    if (!p || !out) return pool_bad(p, "invalid argument");
    PoolLock lock(p);
    return p->pool.count_work(out);
}

const char* sph_pool_last_error(const sph_pool* p)
{
    if (!p) return "null pool";
    return p->pool.err.c_str();
}

}  // extern "C"
