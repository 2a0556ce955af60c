// Kernels of the GB300 SPH particle loop.  Each kernel names the reference
// pass (josemanuel28v/SPH, src/...) whose arithmetic it performs; the grid
// build replaces the reference's unordered_map hash grid (HashTable.h) with a
// counting sort of particles by cell key.
//
// Particle state is kept in cell order (SoA), re-sorted every grid build;
// id[] maps a sorted slot back to the particle's original index, and within a
// cell particles are ordered by id, which is the reference's insertion order
// (SPHSolver.cpp:188-191), so every neighbour sum visits candidates in the
// reference's order.
#pragma once

#include "sph_device.cuh"

#include <cuda_fp16.h>

namespace sph {

template <typename R> struct Fluid {
    P4<R>* pos;      // xyz: position (FP64: absolute; FP32: offset from own cell corner)
    P4<R>* vel;      // xyz: velocity; w: density (written by the density pass)
    P4<R>* acc;      // xyz: non-pressure acceleration
    P4<R>* xk;       // per-pass copy of position with a scalar in w
    P4<R>* predR;    // PCISPH predicted position (same frame as pos)
    P4<R>* predV;    // PCISPH predicted velocity
    P4<R>* pacc;     // PCISPH pressure acceleration
    P4<R>* normal;   // surface-tension normals
    R* rho;
    R* alpha;
    R* pred;         // DFSPH predicted density
    R* div;          // DFSPH divergence error
    R* press;
    R* kappa;        // DFSPH density warm-start accumulator (k)
    R* kappav;       // DFSPH divergence accumulator (kv)
    uint32_t* cell;  // packed cell coordinates
    uint32_t* id;    // original particle index
    uint32_t n;      // particle slots: launch bound and pair-list stride
    // Scenes with emitters: the active particle count on the device (slots
    // [0, *na) hold particles; emission appends).  nullptr: all n slots.
    const uint32_t* na;
    __device__ __forceinline__ uint32_t count() const { return na ? *na : n; }
};

template <typename R> struct Boundary {
    P4<R>* pos;      // xyz: position (frame as fluid); w: solver weight (density0 * psi or the model's mass)
    R* psi;
    uint32_t* cell;
    uint32_t* id;
    uint32_t n;
    // PCISPH boundary model (two-way): normals, densities, pressures and
    // p / rho^2 for the pressure walks (null for the Akinci model)
    P4<R>* nrm;
    R *dens, *press, *dp;
};

constexpr unsigned kBlock = 128;

__device__ __forceinline__ unsigned gtid() { return blockIdx.x * blockDim.x + threadIdx.x; }

template <int G, typename T> __device__ __forceinline__ T group_sum(T v)
{
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
template <int G, typename R> __device__ __forceinline__ V3<R> group_sum3(V3<R> v)
{
    return {group_sum<G>(v.x), group_sum<G>(v.y), group_sum<G>(v.z)};
}

// ===========================================================================
// Upload / download
// ===========================================================================

// A particle left the grid box and was kept in a border cell: the sticky
// status bit, and the flag the host reads to grow the box.
__device__ __forceinline__ void flag_out_of_grid(DevScalars* sc)
{
    atomicOr(&sc->status, (unsigned)ST_OUT_OF_GRID);
    sc->escaped = 1u;
}

// One particle from FP64 host-layout position and velocity into slot i of
// the device layout (FP32: offset from the clamped cell's corner), with the
// per-particle solver state zeroed.
template <typename R>
__device__ __forceinline__ void store_particle(const Fluid<R>& f, uint32_t i, double px, double py, double pz, double vx,
                                               double vy, double vz, const GridView& g, double h, DevScalars* sc)
{
    int cx = (int)floor(px / h) - g.ox, cy = (int)floor(py / h) - g.oy, cz = (int)floor(pz / h) - g.oz;
    const int ccx = min(max(cx, 0), g.nx - 1), ccy = min(max(cy, 0), g.ny - 1), ccz = min(max(cz, 0), g.nz - 1);
    if (ccx != cx || ccy != cy || ccz != cz) flag_out_of_grid(sc);
    P4<R> p;
    if constexpr (sizeof(R) == 4) {
        p = {(R)(px - (double)(ccx + g.ox) * h), (R)(py - (double)(ccy + g.oy) * h), (R)(pz - (double)(ccz + g.oz) * h), 0};
    } else {
        p = {(R)px, (R)py, (R)pz, 0};
    }
    f.pos[i] = p;
    f.vel[i] = P4<R>{(R)vx, (R)vy, (R)vz, 0};
    f.acc[i] = P4<R>{0, 0, 0, 0};
    f.kappa[i] = 0;
    f.kappav[i] = 0;
    f.press[i] = 0;
    f.cell[i] = pack_cell(ccx, ccy, ccz);
    f.id[i] = i;
}

// Shifts packed cell indices by whole cells (a grid box re-planned around
// the same cell lattice: cell (x, y, z) of the old box is (x + sx, y + sy,
// z + sz) of the new one).
static __global__ void k_shift_cells(uint32_t n, const uint32_t* __restrict__ na, uint32_t* __restrict__ cell, int sx,
                                     int sy, int sz)
{
    const uint32_t i = gtid();
    if (i >= (na ? *na : n)) return;
    const uint32_t c = cell[i];
    cell[i] = pack_cell(cell_x(c) + sx, cell_y(c) + sy, cell_z(c) + sz);
}

// Host positions (FP64, xyz per particle) into the device layout.
template <typename R>
__global__ void k_upload_fluid(const double* __restrict__ x, const double* __restrict__ v, uint32_t n,
                               uint32_t first, Fluid<R> f, GridView g, double h, DevScalars* sc)
{
    const uint32_t t = gtid();
    if (t >= n) return;
    store_particle(f, first + t, x[3 * t], x[3 * t + 1], x[3 * t + 2], v[3 * t], v[3 * t + 1], v[3 * t + 2], g, h, sc);
}

template <typename R>
__global__ void k_upload_boundary(const double* __restrict__ x, uint32_t n, Boundary<R> b, GridView g, double h,
                                  DevScalars* sc)
{
    const uint32_t i = gtid();
    if (i >= n) return;
    const double px = x[3 * i], py = x[3 * i + 1], pz = x[3 * i + 2];
    int cx = (int)floor(px / h) - g.ox, cy = (int)floor(py / h) - g.oy, cz = (int)floor(pz / h) - g.oz;
    const int ccx = min(max(cx, 0), g.nx - 1), ccy = min(max(cy, 0), g.ny - 1), ccz = min(max(cz, 0), g.nz - 1);
    if (ccx != cx || ccy != cy || ccz != cz) flag_out_of_grid(sc);
    if constexpr (sizeof(R) == 4)
        b.pos[i] = {(R)(px - (double)(ccx + g.ox) * h), (R)(py - (double)(ccy + g.oy) * h), (R)(pz - (double)(ccz + g.oz) * h), 0};
    else
        b.pos[i] = {(R)px, (R)py, (R)pz, 0};
    b.cell[i] = pack_cell(ccx, ccy, ccz);
    b.id[i] = i;
}

// Absolute FP64 position of a stored point.
template <typename R>
__device__ __forceinline__ void abs_pos(const P4<R>& p, uint32_t c, const GridView& g, double h, double* out)
{
    if constexpr (sizeof(R) == 4) {
        out[0] = (double)(cell_x(c) + g.ox) * h + (double)p.x;
        out[1] = (double)(cell_y(c) + g.oy) * h + (double)p.y;
        out[2] = (double)(cell_z(c) + g.oz) * h + (double)p.z;
    } else {
        out[0] = p.x; out[1] = p.y; out[2] = p.z;
    }
}

// Sorted-order field -> original order, FP64.  kind: 0 vector, 1 position
// (converted to absolute coordinates), 2 scalar, 3 w component.
template <typename R>
__global__ void k_download(uint32_t n, const P4<R>* __restrict__ v4, const R* __restrict__ s, const uint32_t* __restrict__ id,
                           const uint32_t* __restrict__ cell, GridView g, double h, int kind, double* __restrict__ out)
{
    const uint32_t i = gtid();
    if (i >= n) return;
    const uint32_t o = id[i];
    if (kind == 2) { out[o] = (double)s[i]; return; }
    const P4<R> p = v4[i];
    if (kind == 3) { out[o] = (double)p.w; return; }
    if (kind == 1) {
        double a[3];
        abs_pos(p, cell[i], g, h, a);
        out[3 * o] = a[0]; out[3 * o + 1] = a[1]; out[3 * o + 2] = a[2];
    } else {
        out[3 * o] = (double)p.x; out[3 * o + 1] = (double)p.y; out[3 * o + 2] = (double)p.z;
    }
}

// ===========================================================================
// Grid build: cell update -> count -> scan -> scatter -> in-cell id order
// ===========================================================================

// The z offset in the frame of the cell's z index modulo 3, in [0, 3h) for
// an in-grid particle: the FP32 list build's half-precision cull reads the
// z distance of a candidate in cells z-1..z+1 from it without the
// candidate's cell (kept in position.w, which fluid positions leave unused).
__device__ __forceinline__ float zframe3(float oz, int cz, float h) { return oz + (float)(cz % 3) * h; }

// Moves particles (MOVE: x += v dt, DFSPHSolver::updatePositions
// DFSPHSolver.cpp:216-236), recomputes their cells (HashTable.h:81) and
// counts them per cell key.
template <typename R, bool MOVE, bool KEY = true>
__global__ void k_cell_update(uint32_t n, P4<R>* __restrict__ pos, const P4<R>* __restrict__ vel, uint32_t* __restrict__ cell,
                              uint32_t* __restrict__ key, uint32_t* __restrict__ slot, uint32_t* __restrict__ count,
                              GridView g, R h, double hd, DevScalars* sc, uint32_t* __restrict__ cell_epoch = nullptr,
                              P4<R>* __restrict__ carry = nullptr, const uint32_t* __restrict__ na = nullptr)
{
    const uint32_t i = gtid();
    if (i >= (na ? *na : n)) return;
    P4<R> p = pos[i];
    if (MOVE) {
        const R dt = (R)sc->dt;
        const P4<R> v = vel[i];
        p.x = p.x + v.x * dt; p.y = p.y + v.y * dt; p.z = p.z + v.z * dt;
    }
    // a NaN / Inf position (or, moved, velocity) never meets a neighbour, so
    // no solver sum would notice it (as in the reference): flag it here
    if (!(isfinite(p.x) && isfinite(p.y) && isfinite(p.z))) atomicOr(&sc->status, (unsigned)ST_NONFINITE);
    const uint32_t c0 = cell[i];
    int cx, cy, cz;
    if constexpr (sizeof(R) == 4) {
        const int x0 = cell_x(c0), y0 = cell_y(c0), z0 = cell_z(c0);
        const int sx = (int)floorf(p.x / h), sy = (int)floorf(p.y / h), sz = (int)floorf(p.z / h);
        cx = x0 + sx; cy = y0 + sy; cz = z0 + sz;
        const int ccx = min(max(cx, 0), g.nx - 1), ccy = min(max(cy, 0), g.ny - 1), ccz = min(max(cz, 0), g.nz - 1);
        if (ccx != cx || ccy != cy || ccz != cz) flag_out_of_grid(sc);
        p.x -= (R)(ccx - x0) * h; p.y -= (R)(ccy - y0) * h; p.z -= (R)(ccz - z0) * h;
        if (carry) {  // a second point stored in the particle's frame (PCISPH predicted position)
            P4<R> q = carry[i];
            q.x -= (R)(ccx - x0) * h; q.y -= (R)(ccy - y0) * h; q.z -= (R)(ccz - z0) * h;
            carry[i] = q;
        }
        // keep in-grid offsets inside [0, h) so the 27-cell walk covers the support
        if (ccx == cx) p.x = fminf(fmaxf(p.x, 0.f), __int_as_float(__float_as_int(h) - 1));
        if (ccy == cy) p.y = fminf(fmaxf(p.y, 0.f), __int_as_float(__float_as_int(h) - 1));
        if (ccz == cz) p.z = fminf(fmaxf(p.z, 0.f), __int_as_float(__float_as_int(h) - 1));
        p.w = zframe3(p.z, ccz, h);
        cx = ccx; cy = ccy; cz = ccz;
    } else {
        cx = (int)floor((double)p.x / hd) - g.ox;
        cy = (int)floor((double)p.y / hd) - g.oy;
        cz = (int)floor((double)p.z / hd) - g.oz;
        const int ccx = min(max(cx, 0), g.nx - 1), ccy = min(max(cy, 0), g.ny - 1), ccz = min(max(cz, 0), g.nz - 1);
        if (ccx != cx || ccy != cy || ccz != cz) flag_out_of_grid(sc);
        cx = ccx; cy = ccy; cz = ccz;
    }
    pos[i] = p;
    cell[i] = pack_cell(cx, cy, cz);
    if (!KEY) return;  // positions and cells only (the PCISPH boundary corrections follow)
    const uint32_t k = cell_key(g, cx, cy, cz);
    if (cell_epoch) atomicMin(cell_epoch + k, sc->grid_epoch);  // the cell exists from this build on
    key[i] = k;
    slot[i] = atomicAdd(count + k, 1u);
}

// Same for static points (boundary): cells already known.
static __global__ void k_cell_count(uint32_t n, const uint32_t* __restrict__ cell, uint32_t* __restrict__ key,
                             uint32_t* __restrict__ slot, uint32_t* __restrict__ count, GridView g)
{
    const uint32_t i = gtid();
    if (i >= n) return;
    const uint32_t c = cell[i];
    const uint32_t k = cell_key(g, cell_x(c), cell_y(c), cell_z(c));
    key[i] = k;
    slot[i] = atomicAdd(count + k, 1u);
}

// Exclusive scan of the per-key counts into cell starts (three phases:
// per-tile scan with warp shuffles, scan of tile sums, add).  Counts are
// zeroed for the next build.
constexpr unsigned kScanThreads = 256, kScanPer = 8, kScanTile = kScanThreads * kScanPer;

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v)
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* sh, uint32_t* total)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const uint32_t inc = warp_incl_scan(v);
    if (lane == 31) sh[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        const uint32_t w = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0u;
        const uint32_t wi = warp_incl_scan(w);
        sh[lane] = wi - w;
        if (lane == 31) sh[32] = wi;
    }
    __syncthreads();
    const uint32_t r = inc - v + sh[wid];
    *total = sh[32];
    __syncthreads();
    return r;
}

// Each thread owns PER consecutive keys moved as 16-byte vectors when the
// run lies inside the key range (count and starts are 256-byte aligned
// allocations and PER is a multiple of 4, so every run is 16-byte aligned).
// PER (the scan width) is a tuning parameter of the pool; the result does
// not depend on it.
template <unsigned PER = kScanPer>
static __global__ void __launch_bounds__(kScanThreads) k_scan_tiles(uint32_t nkeys, uint32_t* __restrict__ count,
                                                             uint32_t* __restrict__ starts, uint32_t* __restrict__ tile_sums)
{
    static_assert(PER % 4 == 0, "whole uint4 per thread");
    __shared__ uint32_t sh[33];
    const uint32_t base = blockIdx.x * (kScanThreads * PER) + threadIdx.x * PER;
    uint32_t v[PER];
    const bool full = base + PER <= nkeys;
    if (full) {
        uint4* c4 = reinterpret_cast<uint4*>(count + base);
#pragma unroll
        for (unsigned q = 0; q < PER / 4; ++q) {
            const uint4 a = c4[q];
            v[4 * q] = a.x; v[4 * q + 1] = a.y; v[4 * q + 2] = a.z; v[4 * q + 3] = a.w;
            c4[q] = make_uint4(0u, 0u, 0u, 0u);
        }
    } else {
#pragma unroll
        for (unsigned k = 0; k < PER; ++k) {
            const uint32_t idx = base + k;
            v[k] = idx < nkeys ? count[idx] : 0u;
            if (idx < nkeys) count[idx] = 0u;
        }
    }
    uint32_t s = 0;
#pragma unroll
    for (unsigned k = 0; k < PER; ++k) s += v[k];
    uint32_t total;
    uint32_t run = block_excl_scan(s, sh, &total);
#pragma unroll
    for (unsigned k = 0; k < PER; ++k) {
        const uint32_t t = v[k];
        v[k] = run;
        run += t;
    }
    if (full) {
        uint4* s4 = reinterpret_cast<uint4*>(starts + base);
#pragma unroll
        for (unsigned q = 0; q < PER / 4; ++q) s4[q] = make_uint4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
    } else {
#pragma unroll
        for (unsigned k = 0; k < PER; ++k)
            if (base + k < nkeys) starts[base + k] = v[k];
    }
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

static __global__ void __launch_bounds__(1024) k_scan_tile_sums(uint32_t ntiles, uint32_t* __restrict__ tile_sums,
                                                         uint32_t* __restrict__ starts, uint32_t nkeys)
{
    __shared__ uint32_t sh[33];
    uint32_t carry = 0;
    for (uint32_t b = 0; b < ntiles; b += blockDim.x) {
        const uint32_t idx = b + threadIdx.x;
        const uint32_t v = idx < ntiles ? tile_sums[idx] : 0u;
        uint32_t total;
        const uint32_t ex = block_excl_scan(v, sh, &total);
        if (idx < ntiles) tile_sums[idx] = ex + carry;
        carry += total;
    }
    if (threadIdx.x == 0) starts[nkeys] = carry;
}

template <unsigned PER = kScanPer>
static __global__ void __launch_bounds__(kScanThreads) k_scan_add(uint32_t nkeys, const uint32_t* __restrict__ tile_sums,
                                                           uint32_t* __restrict__ starts)
{
    const uint32_t add = tile_sums[blockIdx.x];
    const uint32_t base = blockIdx.x * (kScanThreads * PER) + threadIdx.x * PER;
    if (base + PER <= nkeys) {
        uint4* s4 = reinterpret_cast<uint4*>(starts + base);
#pragma unroll
        for (unsigned q = 0; q < PER / 4; ++q) {
            uint4 a = s4[q];
            a.x += add; a.y += add; a.z += add; a.w += add;
            s4[q] = a;
        }
    } else {
        for (uint32_t k = 0; k < PER; ++k)
            if (base + k < nkeys) starts[base + k] += add;
    }
}

static __global__ void k_scatter(uint32_t n, const uint32_t* __restrict__ key, const uint32_t* __restrict__ slot,
                          const uint32_t* __restrict__ starts, uint32_t* __restrict__ tmp, const uint32_t* __restrict__ na = nullptr)
{
    const uint32_t i = gtid();
    if (i >= (na ? *na : n)) return;
    tmp[starts[key[i]] + slot[i]] = i;
}

// Final slot of the particle at tmp position p: its cell start plus the
// number of particles of the same cell with a smaller id.
__device__ __forceinline__ uint32_t final_slot(uint32_t p, const uint32_t* __restrict__ tmp, const uint32_t* __restrict__ key,
                                               const uint32_t* __restrict__ id, const uint32_t* __restrict__ starts,
                                               uint32_t* src_out)
{
    const uint32_t i = tmp[p];
    const uint32_t k = key[i];
    const uint32_t s = starts[k], e = starts[k + 1];
    const uint32_t me = id[i];
    uint32_t rank = 0;
    for (uint32_t q = s; q < e; ++q) rank += (id[tmp[q]] < me) ? 1u : 0u;
    *src_out = i;
    return s + rank;
}

// Gather of the state that survives a re-sort (x, v, DFSPH k, kv and the
// last predicted density; the other fields are recomputed after every build).
// posh (FP32, optional): also the half-precision copy of the positions the
// list build culls with, two particles (2k, 2k+1) per 16-byte word:
// {x pair, y pair, z pair, unused} as half2, z in the cell's modulo-3 frame
// (position.w, written by the cell update).
template <typename R>
__global__ void k_gather_fluid(uint32_t n, const uint32_t* __restrict__ tmp, const uint32_t* __restrict__ key,
                               const uint32_t* __restrict__ starts, Fluid<R> src, Fluid<R> dst,
                               uint4* __restrict__ posh = nullptr)
{
    const uint32_t p = gtid();
    if (p >= src.count()) return;
    uint32_t i;
    const uint32_t d = final_slot(p, tmp, key, src.id, starts, &i);
    const P4<R> x = src.pos[i];
    dst.pos[d] = x;
    if constexpr (sizeof(R) == 4) {
        if (posh) {
            __half* ph = reinterpret_cast<__half*>(posh) + (size_t)(d >> 1) * 8 + (d & 1);
            ph[0] = __float2half_rn(x.x);
            ph[2] = __float2half_rn(x.y);
            ph[4] = __float2half_rn(x.w);
        }
    }
    dst.vel[d] = src.vel[i];
    dst.kappa[d] = src.kappa[i];
    dst.kappav[d] = src.kappav[i];
    dst.pred[d] = src.pred[i];
    dst.cell[d] = src.cell[i];
    dst.id[d] = src.id[i];
    // PCISPH boundary model: a particle's normal from its last collision is
    // read by the next step's velocity correction (double-buffered then)
    if (src.normal != dst.normal) dst.normal[d] = src.normal[i];
}

template <typename R>
__global__ void k_gather_boundary(uint32_t n, const uint32_t* __restrict__ tmp, const uint32_t* __restrict__ key,
                                  const uint32_t* __restrict__ starts, Boundary<R> src, Boundary<R> dst)
{
    const uint32_t p = gtid();
    if (p >= n) return;
    uint32_t i;
    const uint32_t d = final_slot(p, tmp, key, src.id, starts, &i);
    dst.pos[d] = src.pos[i];
    dst.cell[d] = src.cell[i];
    dst.id[d] = src.id[i];
    if (src.nrm) dst.nrm[d] = src.nrm[i];
}

// ===========================================================================
// Neighbour walks
// ===========================================================================

// AkinciBoundaryModel::computeVolume AkinciBoundayModel.cpp:11-40:
// psi_b = 1 / sum_{b'} W(x_b - x_b') over the boundary candidates.
template <typename R>
__global__ void k_boundary_psi(Boundary<R> b, GridView g, const uint32_t* __restrict__ bstarts, Consts<R> c)
{
    const uint32_t i = gtid();
    if (i >= b.n) return;
    const P4<R> pi = b.pos[i];
    R delta = 0;
    walk<R, 1>(g, bstarts, b.cell[i], xyz(pi), c.h, 0, [&](uint32_t j, V3<R> s) {
        const V3<R> r = s - xyz(ldg4(b.pos + j));
        const R r2 = dot3(r, r);
        if (r2 <= c.cull2) delta += cubic_W(c, sqrt(r2));
    });
    const R psi = (R)1 / delta;
    b.psi[i] = psi;
    b.pos[i].w = c.density0 * psi;
}

// ---------------------------------------------------------------------------
// PCISPH / WCSPH candidate lists (one lane per particle).  The reference's
// PCISPH and WCSPH sums run over the particles of the 27 cells found at the
// start of the step (HashTable::neighborhoodSearch, HashTable.h:136-170), at
// the current positions (densities, normals, non-pressure forces, pressure
// accelerations, WCSPH's pressure force) or the predicted ones (PCISPH's
// predicted densities).  The density pass records, once per step, every
// fluid candidate of the 27 cells whose current distance is within
// REACH = h + margin, in the walk's order, with its cell offset; the later
// passes visit the list instead of the cells.
// A candidate left out lies beyond h at the current positions, and beyond h
// at the predicted ones while every predicted displacement stays below
// margin / 2 (checked per loop iteration; otherwise the predicted-density
// pass walks the cells): its terms are the ones the walks skip, so the sums
// are the same, bit for bit.  A particle with more than kmax candidates
// walks the cells.
constexpr uint32_t kCandIdxBits = 27;
constexpr uint32_t kCandIdxMask = (1u << kCandIdxBits) - 1u;

struct CandLists {
    const uint32_t* idx;   // kmax * n, slot-major: j | (cell offset code << 27); nullptr: no lists
    const uint32_t* cnt;   // candidates per particle (may exceed kmax)
    uint32_t kmax;
    unsigned* fault;       // status word of the bounds-checked build (SPH_INDEX_OK)
    __device__ __forceinline__ bool has(uint32_t i) const { return idx && cnt[i] <= kmax; }
};

// walk<R, 1> (rolled out, cells within reach2 of the particle), passing each
// candidate's cell offset code (dx + 1) * 9 + (dy + 1) * 3 + (dz + 1).
template <typename R, typename F>
__device__ __forceinline__ void walk_reach(const GridView& g, const uint32_t* __restrict__ starts, uint32_t pc, V3<R> xi,
                                           R h, R reach2, F&& f)
{
    constexpr bool REL = sizeof(R) == 4;
    const int cx = cell_x(pc), cy = cell_y(pc), cz = cell_z(pc);
    const int z0 = cz > 0 ? cz - 1 : 0;
    const int z1 = cz + 1 < g.nz ? cz + 1 : g.nz - 1;
    const R ofx = REL ? xi.x : xi.x - (R)(cx + g.ox) * h;
    const R ofy = REL ? xi.y : xi.y - (R)(cy + g.oy) * h;
    const R ofz = REL ? xi.z : xi.z - (R)(cz + g.oz) * h;
    const R gxm = ofx > (R)0 ? ofx * ofx : (R)0, gxp = h - ofx > (R)0 ? (h - ofx) * (h - ofx) : (R)0;
    const R gym = ofy > (R)0 ? ofy * ofy : (R)0, gyp = h - ofy > (R)0 ? (h - ofy) * (h - ofy) : (R)0;
    const R gzm = ofz > (R)0 ? ofz * ofz : (R)0, gzp = h - ofz > (R)0 ? (h - ofz) * (h - ofz) : (R)0;
    const R lim = reach2 * (R)(1.0 + 1e-5);
    const R szm = xi.z + h, sz0 = xi.z, szp = xi.z - h;
#pragma unroll 1
    for (int c = 0; c < 9; ++c) {
        const int dx = c / 3 - 1, dy = c % 3 - 1;
        const int x = cx + dx, y = cy + dy;
        const R gxy = (dx < 0 ? gxm : (dx > 0 ? gxp : (R)0)) + (dy < 0 ? gym : (dy > 0 ? gyp : (R)0));
        if (x < 0 || x >= g.nx || y < 0 || y >= g.ny || !(gxy <= lim)) continue;
        const uint32_t base = (__ldg(g.mortx + x) | __ldg(g.morty + y)) * (uint32_t)g.nz;
        const uint32_t s0 = __ldg(starts + base + z0), sm = __ldg(starts + base + cz);
        const uint32_t sp = __ldg(starts + base + cz + 1), s1 = __ldg(starts + base + z1 + 1);
        const uint32_t bb = gxy + gzm <= lim ? s0 : sm, ee = gxy + gzp <= lim ? s1 : sp;
        V3<R> s = REL ? V3<R>{xi.x - (R)dx * h, xi.y - (R)dy * h, xi.z} : xi;
#pragma unroll 1
        for (uint32_t j = bb; j < ee; ++j) {
            const int dz = j < sm ? -1 : (j < sp ? 0 : 1);
            if (REL) s.z = dz < 0 ? szm : (dz == 0 ? sz0 : szp);
            f(j, s, (uint32_t)(c * 3 + dz + 1));
        }
    }
}

// The listed candidates of particle i, with the same shifted position s as
// the cell walk passes for them.
template <typename R, typename F>
__device__ __forceinline__ void list_visit(const CandLists& L, uint32_t n, uint32_t i, V3<R> xi, R h, F&& f)
{
    constexpr bool REL = sizeof(R) == 4;
    const uint32_t cnt = L.cnt[i];
    const R szm = xi.z + h, sz0 = xi.z, szp = xi.z - h;
#pragma unroll 1
    for (uint32_t k = 0; k < cnt; ++k) {
        const uint32_t e = __ldg(L.idx + (size_t)k * n + i);
        const uint32_t code = e >> kCandIdxBits;
        const int dx = (int)(code / 9) - 1, dy = (int)((code / 3) % 3) - 1, dz = (int)(code % 3) - 1;
        const V3<R> s = REL ? V3<R>{xi.x - (R)dx * h, xi.y - (R)dy * h, dz < 0 ? szm : (dz == 0 ? sz0 : szp)} : xi;
        const uint32_t j = e & kCandIdxMask;
        if (!SPH_INDEX_OK(j, n, L.fault)) continue;
        f(j, s);
    }
}

// Fluid candidates of particle i at lane LANE of G: the list (G = 1 and a
// stored list) or the cell walk.
template <typename R, int G, bool TRIM = true, typename F>
__device__ __forceinline__ void fluid_visit(const CandLists& L, uint32_t n, uint32_t i, const GridView& g,
                                            const uint32_t* __restrict__ cs, uint32_t pc, V3<R> xi, R h, int lane, F&& f)
{
    if (G == 1 && L.has(i)) list_visit<R>(L, n, i, xi, h, f);
    else walk<R, G, TRIM>(g, cs, pc, xi, h, lane, f);
}

// Densities (SPHSolver::computeFluidDensities SPHSolver.cpp:44-91, as
// k_density<R, 1, false, EOS>, EOS: with WCSPH's equation of state) fused
// with the candidate lists' build.
template <typename R, bool EOS = false>
__global__ void __launch_bounds__(kBlock) k_density_cand(Fluid<R> f, const P4<R>* __restrict__ bpos, GridView g,
                                                         const uint32_t* __restrict__ cs, const uint32_t* __restrict__ bs,
                                                         Consts<R> c, int akinci, R reach2, uint32_t* __restrict__ idx,
                                                         uint32_t* __restrict__ cnt, uint32_t kmax)
{
    const uint32_t i = gtid();
    if (i >= f.count()) return;
    const uint32_t n = f.n;
    const V3<R> xi = xyz(f.pos[i]);
    const uint32_t pc = f.cell[i];
    R density = 0;
    uint32_t m = 0;
    walk_reach<R>(g, cs, pc, xi, c.h, reach2, [&](uint32_t j, V3<R> s, uint32_t code) {
        const V3<R> r = s - xyz(ldg4(f.pos + j));
        const R r2 = dot3(r, r);
        if (r2 <= reach2) {
            if (m < kmax) idx[(size_t)m * n + i] = j | (code << kCandIdxBits);
            ++m;
        }
        if (r2 <= c.cull2) density += c.mass * cubic_W(c, sqrt(r2));
    });
    if (akinci)
        walk<R, 1>(g, bs, pc, xi, c.h, 0, [&](uint32_t j, V3<R> s) {
            const P4<R> pb = ldg4(bpos + j);
            const V3<R> r = s - xyz(pb);
            const R r2 = dot3(r, r);
            if (r2 <= c.cull2) density += pb.w * cubic_W(c, sqrt(r2));
        });
    f.rho[i] = density;
    f.vel[i].w = density;
    cnt[i] = m;
    if (EOS) {  // as k_density<R, G, false, true>
        const R p = fmax((R)0, c.k_eos * (pow(density / c.density0, c.gamma) - (R)1));
        f.press[i] = p;
        f.xk[i] = P4<R>{xi.x, xi.y, xi.z, p / (density * density)};
    }
}

// SPHSolver::computeFluidDensities SPHSolver.cpp:44-91, fused with
// DFSPHSolver::computeAlpha DFSPHSolver.cpp:114-189 (ALPHA) or the Tait
// equation of state WCSPHSolver::computeFluidPressures WCSPHSolver.cpp:80-95
// (EOS, which also stores p / rho^2 for the pressure-force walk).
template <typename R, int G, bool ALPHA, bool EOS>
__global__ void __launch_bounds__(kBlock) k_density(Fluid<R> f, const P4<R>* __restrict__ bpos, GridView g,
                                                    const uint32_t* __restrict__ cs, const uint32_t* __restrict__ bs,
                                                    Consts<R> c, int akinci)
{
    const uint32_t t = gtid();
    const uint32_t i = t / G;
    const int lane = (int)(t % G);
    const bool valid = i < f.count();
    R density = 0, sumSq = 0;
    V3<R> sumGrad = {0, 0, 0};
    V3<R> xi = {0, 0, 0};
    if (valid) {
        const P4<R> pi = f.pos[i];
        xi = xyz(pi);
        const uint32_t pc = f.cell[i];
        walk<R, G>(g, cs, pc, xi, c.h, lane, [&](uint32_t j, V3<R> s) {
            const V3<R> r = s - xyz(ldg4(f.pos + j));
            const R r2 = dot3(r, r);
            if (r2 <= c.cull2) {
                density += c.mass * cubic_W(c, sqrt(r2));
                if (ALPHA) {
                    const V3<R> mg = c.mass * cubic_gradW(c, r, r2);
                    sumGrad = sumGrad + mg;
                    if constexpr (sizeof(R) == 8) {
                        const R m = sqrt(dot3(mg, mg));
                        sumSq += m * m;
                    } else {
                        sumSq += dot3(mg, mg);
                    }
                }
            }
        });
        if (akinci)
            walk<R, G>(g, bs, pc, xi, c.h, lane, [&](uint32_t j, V3<R> s) {
                const P4<R> pb = ldg4(bpos + j);
                const V3<R> r = s - xyz(pb);
                const R r2 = dot3(r, r);
                if (r2 <= c.cull2) {
                    density += pb.w * cubic_W(c, sqrt(r2));
                    if (ALPHA) sumGrad = sumGrad + pb.w * cubic_gradW(c, r, r2);
                }
            });
    }
    if (G > 1) {
        density = group_sum<G>(density);
        if (ALPHA) { sumGrad = group_sum3<G>(sumGrad); sumSq = group_sum<G>(sumSq); }
    }
    if (!valid || lane != 0) return;
    f.rho[i] = density;
    f.vel[i].w = density;
    if (ALPHA) {
        R den;
        if constexpr (sizeof(R) == 8) {
            const R m = sqrt(dot3(sumGrad, sumGrad));
            den = m * m + sumSq;
        } else {
            den = dot3(sumGrad, sumGrad) + sumSq;
        }
        f.alpha[i] = (fabs(den) > c.eps) ? density / den : (R)0;
    }
    if (EOS) {
        const R p = fmax((R)0, c.k_eos * (pow(density / c.density0, c.gamma) - (R)1));
        f.press[i] = p;
        f.xk[i] = P4<R>{xi.x, xi.y, xi.z, p / (density * density)};
    }
}

// WCSPHSolver::computePressureForce WCSPHSolver.cpp:132-188 (xk.w = p/rho^2)
template <typename R, int G>
__global__ void __launch_bounds__(kBlock) k_wcsph_pressure_force(Fluid<R> f, const P4<R>* __restrict__ bpos, GridView g,
                                                                 const uint32_t* __restrict__ cs, const uint32_t* __restrict__ bs,
                                                                 Consts<R> c, int akinci, const R* __restrict__ bdp,
                                                                 CandLists L = CandLists{nullptr, nullptr, 0u})
{
    const uint32_t t = gtid();
    const uint32_t i = t / G;
    const int lane = (int)(t % G);
    const bool valid = i < f.count();
    V3<R> sum = {0, 0, 0};
    if (valid) {
        const P4<R> pi = f.xk[i];
        const V3<R> xi = xyz(pi);
        const R dpi = pi.w;
        const uint32_t pc = f.cell[i];
        fluid_visit<R, G>(L, f.n, i, g, cs, pc, xi, c.h, lane, [&](uint32_t j, V3<R> s) {
            const P4<R> pj = ldg4(f.xk + j);
            const V3<R> r = s - xyz(pj);
            const R r2 = dot3(r, r);
            if (r2 <= c.cull2) sum = sum - (c.mass * (dpi + pj.w)) * cubic_gradW(c, r, r2);
        });
        if (akinci)
            walk<R, G>(g, bs, pc, xi, c.h, lane, [&](uint32_t j, V3<R> s) {
                const P4<R> pb = ldg4(bpos + j);
                const V3<R> r = s - xyz(pb);
                const R r2 = dot3(r, r);
                // Akinci: rho0 psi_b (p_i / rho_i^2); PCISPH model: m_b (p_i / rho_i^2 + p_b / rho_b^2)
                // (WCSPHSolver.cpp:162-186)
                const R q = bdp ? dpi + bdp[j] : dpi * (R)1;
                if (r2 <= c.cull2) sum = sum - (pb.w * q) * cubic_gradW(c, r, r2);
            });
    }
    if (G > 1) sum = group_sum3<G>(sum);
    if (!valid || lane != 0) return;
    P4<R> a = f.acc[i];
    a.x += sum.x; a.y += sum.y; a.z += sum.z;
    f.acc[i] = a;
}

// SurfaceTensionAkinci::step, normal pass SurfaceTensionAkinci.h:43-61: this
// lane's part of particle i's sum (the caller adds the lanes and scales by h).
template <typename R, int G>
__device__ __forceinline__ V3<R> st_normal_sum(uint32_t i, int lane, const Fluid<R>& f, const GridView& g,
                                               const uint32_t* __restrict__ cs, const Consts<R>& c,
                                               const CandLists& L = CandLists{nullptr, nullptr, 0u})
{
    V3<R> ni = {0, 0, 0};
    const V3<R> xi = xyz(f.pos[i]);
    fluid_visit<R, G>(L, f.n, i, g, cs, f.cell[i], xi, c.h, lane, [&](uint32_t j, V3<R> s) {
        const V3<R> r = s - xyz(ldg4(f.pos + j));
        const R r2 = dot3(r, r);
        if (r2 <= c.cull2) {
            const R vol = c.mass / ldg4(f.vel + j).w;
            ni = ni + vol * cubic_gradW(c, r, r2);
        }
    });
    return ni;
}

template <typename R, int G>
__global__ void __launch_bounds__(kBlock) k_st_normals(Fluid<R> f, GridView g, const uint32_t* __restrict__ cs, Consts<R> c,
                                                       CandLists L = CandLists{nullptr, nullptr, 0u})
{
    const uint32_t t = gtid();
    const uint32_t i = t / G;
    const int lane = (int)(t % G);
    const bool valid = i < f.count();
    V3<R> ni = {0, 0, 0};
    if (valid) ni = st_normal_sum<R, G>(i, lane, f, g, cs, c, L);
    if (G > 1) ni = group_sum3<G>(ni);
    if (!valid || lane != 0) return;
    ni = ni * ((R)1 * c.h);
    f.normal[i] = P4<R>{ni.x, ni.y, ni.z, 0};
}

// This lane's parts of particle i's non-pressure forces, each accumulated
// separately (av fluid viscosity, avb boundary viscosity, ast surface
// tension, aad adhesion) over one fluid and one boundary walk:
//   XSPHViscosity::step XSPHViscosity.h:32-69
//   StandardViscosityForce::step StandardViscosityForce.h:29-79
//   ArtificialViscosity::step ArtificialViscosity.h:31-83
//   SurfaceTensionAkinci::step (cohesion + curvature) SurfaceTensionAkinci.h:64-97
//   AdhesionForce::step AdhesionForce.h:30-62
template <typename R> struct NPForces {
    V3<R> av, avb, ast, aad;
};

template <typename R, int G>
__device__ __forceinline__ NPForces<R> npforce_sums(uint32_t i, int lane, const Fluid<R>& f,
                                                    const P4<R>* __restrict__ bpos, const GridView& g,
                                                    const uint32_t* __restrict__ cs, const uint32_t* __restrict__ bs,
                                                    const Consts<R>& c, int akinci, R dt,
                                                    const CandLists& L = CandLists{nullptr, nullptr, 0u})
{
    const int fl = c.force_flags;
    V3<R> av = {0, 0, 0}, avb = {0, 0, 0}, ast = {0, 0, 0}, aad = {0, 0, 0};
    const V3<R> xi = xyz(f.pos[i]);
    const P4<R> vi4 = f.vel[i];
    const V3<R> vi = xyz(vi4);
    const R rho_i = vi4.w;
    V3<R> ni = {0, 0, 0};
    if (fl & F_SURFACE_TENSION) ni = xyz(f.normal[i]);
    const uint32_t pc = f.cell[i];
    const R h2 = c.h * c.h;
    if (fl & (F_XSPH | F_STD_VISC | F_ART_VISC | F_SURFACE_TENSION))
        fluid_visit<R, G>(L, f.n, i, g, cs, pc, xi, c.h, lane, [&](uint32_t j, V3<R> s) {
            const V3<R> r = s - xyz(ldg4(f.pos + j));
            const R r2 = dot3(r, r);
            if (!(r2 <= c.cull2)) return;
            const P4<R> vj4 = ldg4(f.vel + j);
            const V3<R> vj = xyz(vj4);
            const R rho_j = vj4.w;
            const R rl = sqrt(r2);
            if (fl & F_XSPH)
                av = av + (((c.visc * (c.mass / rho_j)) * (vj - vi)) * cubic_W(c, rl)) / dt;
            if (fl & F_STD_VISC)
                av = av + ((c.mass * (vj - vi)) / rho_j) * visc_laplW(c, r2);
            if (fl & F_ART_VISC) {
                const R dotProd = dot3(vi - vj, r);
                const R sqDist = rl * rl;
                const R kij = (R)2 * c.density0 / (rho_i + rho_j);
                av = av + (kij * (R)10 * (R)0.1 * c.visc * (c.mass / rho_j) * dotProd / (sqDist + (R)0.01 * h2)) *
                              cubic_gradW(c, r, r2);
            }
            if (fl & F_SURFACE_TENSION) {
                if (rl > (R)0 && rl <= c.h) {
                    const V3<R> nj = xyz(ldg4(f.normal + j));
                    const R kij = (R)2 * c.density0 / (rho_i + rho_j);
                    const V3<R> coh = ((-c.mass * cohesion_W(c, rl)) * r) / rl;
                    const V3<R> curv = (R)-1 * (ni - nj);
                    ast = ast + (c.st * kij) * (coh + curv);
                }
            }
        });
    const bool bvisc = (fl & F_BVISC) && akinci;
    if ((fl & F_ADHESION) || bvisc)
        walk<R, G>(g, bs, pc, xi, c.h, lane, [&](uint32_t j, V3<R> s) {
            const P4<R> pb = ldg4(bpos + j);
            const V3<R> r = s - xyz(pb);
            const R r2 = dot3(r, r);
            if (!(r2 <= c.cull2)) return;
            const R rl = sqrt(r2);
            if (bvisc) {
                if (fl & F_XSPH)
                    avb = avb + (((c.bvisc * (pb.w / rho_i)) * (-vi)) * cubic_W(c, rl)) / dt;
                if (fl & F_STD_VISC)
                    avb = avb + ((pb.w * (-vi)) / rho_i) * visc_laplW(c, r2);
                if (fl & F_ART_VISC) {
                    const R dotProd = dot3(vi, r);
                    const R sqDist = rl * rl;
                    avb = avb + ((R)10 * (R)0.1 * c.bvisc * (pb.w / rho_i) * dotProd / (sqDist + (R)0.01 * h2)) *
                                    cubic_gradW(c, r, r2);
                }
            }
            if ((fl & F_ADHESION) && rl > (R)0)
                aad = aad - ((c.adh * pb.w * adhesion_W(c, rl)) * r) / rl;
        });
    return NPForces<R>{av, avb, ast, aad};
}

// The forces added to particle i's acceleration in the reference's plugin
// order (viscosity, surface tension, adhesion;
// Simulation::computeNonPressureForces Simulation.cpp:313-323).
template <typename R>
__device__ __forceinline__ void npforce_apply(uint32_t i, const Fluid<R>& f, const Consts<R>& c, NPForces<R> s)
{
    if (c.force_flags & F_STD_VISC) {
        // viscoForce *= visc / density0 (separately for the boundary sum)
        s.av = s.av * (c.visc / c.density0);
        s.avb = s.avb * (c.bvisc / c.density0);
    }
    P4<R> a = f.acc[i];
    V3<R> tot = {a.x, a.y, a.z};
    tot = tot + s.av;
    tot = tot + s.avb;
    tot = tot + s.ast;
    tot = tot + s.aad;
    f.acc[i] = P4<R>{tot.x, tot.y, tot.z, 0};
}

// Non-pressure forces in one walk (npforce_sums), lanes added, then applied.
template <typename R, int G>
__global__ void __launch_bounds__(kBlock) k_npforce(Fluid<R> f, const P4<R>* __restrict__ bpos, GridView g,
                                                    const uint32_t* __restrict__ cs, const uint32_t* __restrict__ bs,
                                                    Consts<R> c, int akinci, const DevScalars* __restrict__ scr,
                                                    CandLists L = CandLists{nullptr, nullptr, 0u})
{
    const uint32_t t = gtid();
    const uint32_t i = t / G;
    const int lane = (int)(t % G);
    const bool valid = i < f.count();
    NPForces<R> s = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    if (valid) s = npforce_sums<R, G>(i, lane, f, bpos, g, cs, bs, c, akinci, (R)scr->dt, L);
    if (G > 1) {
        s.av = group_sum3<G>(s.av); s.avb = group_sum3<G>(s.avb); s.ast = group_sum3<G>(s.ast); s.aad = group_sum3<G>(s.aad);
    }
    if (!valid || lane != 0) return;
    npforce_apply(i, f, c, s);
}

// ===========================================================================
// DFSPH (DFSPHSolver.cpp)
// ===========================================================================

// DFSPHSolver::updateTimeStep DFSPHSolver.cpp:827-870: CFL step from
// max(0.1, sqrt(|v + (a + g) dt|)) (the reference takes the square root of
// the speed) and the +0.1% / -1% rule on the previous solve's iterations.
template <typename R>
__global__ void __launch_bounds__(256) k_dfsph_cfl(Fluid<R> f, Consts<R> c, DevScalars* sc, LoopLimits lim,
                                                   double* partials)
{
    __shared__ double sh[33];
    const uint32_t i = gtid();
    const R dt = (R)sc->dt;
    double m = 0.1;
    if (i < f.count()) {
        const P4<R> v = f.vel[i], a = f.acc[i];
        const V3<R> cur = {v.x + (a.x + c.gx) * dt, v.y + (a.y + c.gy) * dt, v.z + (a.z + c.gz) * dt};
        m = fmax(m, (double)sqrt(sqrt(dot3(cur, cur))));
    }
    double maxVel;
    if (finish_reduction<true>(m, partials, &sc->block_counter, sh, &maxVel) && threadIdx.x == 0) {
        maxVel = fmax(maxVel, 0.1);
        const double ts = sc->dt;
        const double cflTs = lim.cflFactor * 0.4 * 2.0 * lim.particleRadius / maxVel;
        double newTs;
        if (cflTs < ts) newTs = cflTs;
        else if (sc->iterations > 3) newTs = ts * 0.99;
        else newTs = ts * 1.001;
        newTs = fmax(newTs, lim.minTs);
        newTs = fmin(newTs, lim.maxTs);
        sc->dt = newTs;
        sc->maxVel = maxVel;
    }
}

// DFSPHSolver::predictVelocities DFSPHSolver.cpp:191-214 fused with the first
// loop of DFSPHSolver::densityWarmStart DFSPHSolver.cpp:607-613:
// k <- -max(-k/rho, -1e-9)/dt^2, handed to the warm-start walk in xk.w, and
// the accumulator cleared (DFSPHSolver.cpp:679-689).
template <typename R>
__global__ void k_dfsph_predict_v_warm(Fluid<R> f, Consts<R> c, const DevScalars* __restrict__ sc)
{
    const uint32_t i = gtid();
    if (i >= f.count()) return;
    const R dt = (R)sc->dt;
    P4<R> v = f.vel[i];
    const P4<R> a = f.acc[i];
    v.x = v.x + (a.x + c.gx) * dt; v.y = v.y + (a.y + c.gy) * dt; v.z = v.z + (a.z + c.gz) * dt;
    f.vel[i] = v;
    f.acc[i] = P4<R>{0, 0, 0, 0};
    const R dens = f.rho[i];
    const R ts2 = dt * dt;
    const R t = -f.kappa[i] / dens;
    const R mx = t < (R)-0.000000001 ? (R)-0.000000001 : t;
    const R k = -mx / ts2;
    const P4<R> p = f.pos[i];
    f.xk[i] = P4<R>{p.x, p.y, p.z, k};
    f.kappa[i] = 0;
}

// Velocity corrections sharing one walk:
//   MODE 0  DFSPHSolver::densityWarmStart walk DFSPHSolver.cpp:616-677
//   MODE 1  DFSPHSolver::correctDensityError walk DFSPHSolver.cpp:336-395
//   MODE 2  DFSPHSolver::correctDivergenceError walk DFSPHSolver.cpp:520-579
// xk.w holds each particle's k (resp. kv) for this pass.
template <typename R, int G, int MODE>
__global__ void __launch_bounds__(kBlock) k_dfsph_correct(Fluid<R> f, const P4<R>* __restrict__ bpos, GridView g,
                                                          const uint32_t* __restrict__ cs, const uint32_t* __restrict__ bs,
                                                          Consts<R> c, int akinci, const DevScalars* __restrict__ sc)
{
    if (MODE != 0 && !sc->active) return;
    const uint32_t t = gtid();
    const uint32_t i = t / G;
    const int lane = (int)(t % G);
    const bool valid = i < f.count();
    V3<R> sum = {0, 0, 0};
    R ki = 0;
    if (valid) {
        const P4<R> pi = f.xk[i];
        const V3<R> xi = xyz(pi);
        ki = pi.w;
        const uint32_t pc = f.cell[i];
        walk<R, G>(g, cs, pc, xi, c.h, lane, [&](uint32_t j, V3<R> s) {
            const P4<R> pj = ldg4(f.xk + j);
            const R kSum = ki + pj.w;
            if (!(fabs(kSum) > c.eps)) return;
            const V3<R> r = s - xyz(pj);
            const R r2 = dot3(r, r);
            if (r2 <= c.cull2) sum = sum + (c.mass * kSum) * cubic_gradW(c, r, r2);
        });
        const R kb = MODE == 0 ? c.bwarm * ki : ki;
        if (akinci && fabs(kb) > c.eps)
            walk<R, G>(g, bs, pc, xi, c.h, lane, [&](uint32_t j, V3<R> s) {
                const P4<R> pb = ldg4(bpos + j);
                const V3<R> r = s - xyz(pb);
                const R r2 = dot3(r, r);
                if (r2 <= c.cull2) sum = sum + (pb.w * kb) * cubic_gradW(c, r, r2);
            });
    }
    if (G > 1) sum = group_sum3<G>(sum);
    if (!valid || lane != 0) return;
    const R dt = (R)sc->dt;
    if (MODE == 1) f.kappa[i] += (f.pred[i] - c.density0) * f.alpha[i];
    if (MODE == 2) f.kappav[i] += f.div[i] * f.alpha[i];
    P4<R> v = f.vel[i];
    if (MODE == 0) { v.x -= sum.x * dt; v.y -= sum.y * dt; v.z -= sum.z * dt; }
    else { v.x -= dt * sum.x; v.y -= dt * sum.y; v.z -= dt * sum.z; }
    f.vel[i] = v;
}

// DFSPHSolver::predictDensities DFSPHSolver.cpp:238-309 with the average
// error reduction in FP64, plus the next iteration's k in xk.w and the loop
// control of DFSPHSolver::correctDensityError DFSPHSolver.cpp:325-401.
template <typename R, int G, bool INITIAL>
__global__ void __launch_bounds__(kBlock) k_dfsph_predict_density(Fluid<R> f, const P4<R>* __restrict__ bpos, GridView g,
                                                                  const uint32_t* __restrict__ cs, const uint32_t* __restrict__ bs,
                                                                  Consts<R> c, int akinci, DevScalars* sc, LoopLimits lim,
                                                                  double* partials, cudaGraphConditionalHandle cond)
{
    __shared__ double sh[33];
    if (!INITIAL && !sc->active) return;
    const uint32_t t = gtid();
    const uint32_t i = t / G;
    const int lane = (int)(t % G);
    const bool valid = i < f.count();
    R dc = 0;
    V3<R> xi = {0, 0, 0};
    if (valid) {
        xi = xyz(f.pos[i]);
        const V3<R> vi = xyz(f.vel[i]);
        const uint32_t pc = f.cell[i];
        walk<R, G>(g, cs, pc, xi, c.h, lane, [&](uint32_t j, V3<R> s) {
            const V3<R> r = s - xyz(ldg4(f.pos + j));
            const R r2 = dot3(r, r);
            if (r2 <= c.cull2) dc += c.mass * dot3(vi - xyz(ldg4(f.vel + j)), cubic_gradW(c, r, r2));
        });
        if (akinci)
            walk<R, G>(g, bs, pc, xi, c.h, lane, [&](uint32_t j, V3<R> s) {
                const P4<R> pb = ldg4(bpos + j);
                const V3<R> r = s - xyz(pb);
                const R r2 = dot3(r, r);
                if (r2 <= c.cull2) dc += pb.w * dot3(vi, cubic_gradW(c, r, r2));
            });
    }
    if (G > 1) dc = group_sum<G>(dc);
    double err = 0.0;
    if (valid && lane == 0) {
        const R dt = (R)sc->dt;
        const R rho = f.rho[i];
        R pred = rho + dc * dt;
        pred = pred < c.density0 ? c.density0 : pred;
        f.pred[i] = pred;
        const R k = (pred - c.density0) * f.alpha[i] / ((dt * dt) * rho);
        f.xk[i] = P4<R>{xi.x, xi.y, xi.z, k};
        err = rel_error(c, (double)pred - (double)c.density0);
    }
    double total;
    if (finish_reduction<false>(err, partials, &sc->block_counter, sh, &total) && threadIdx.x == 0) {
        const double avg = f.count() ? total / (double)f.count() : 0.0;
        if (!isfinite(avg)) sc->status |= ST_NONFINITE;
        if (INITIAL) {
            sc->iterations = 0;
            sc->avgDensError = avg;
            sc->active = (lim.minIt > 0u) && (lim.maxIt > 0u);
            if (!sc->active) sc->avgDensError = 0.0;
        } else {
            const unsigned it = ++sc->iterations;
            sc->avgDensError = avg;
            const unsigned act = ((avg > lim.maxError) || (it < lim.minIt)) && (it < lim.maxIt);
            sc->active = act;
            if (!act) {
                sc->sumIterations += it;
                if (it >= lim.maxIt && avg > lim.maxError) sc->status |= ST_ITER_CAP;
            }
        }
        if (cond) cudaGraphSetConditional(cond, sc->active);
    }
}

// DFSPHSolver::computeDivergenceError DFSPHSolver.cpp:408-492 with the loop
// control of DFSPHSolver::correctDivergenceError DFSPHSolver.cpp:505-585
// (bounded by maxIterations, as the reference writes it).
template <typename R, int G, bool INITIAL>
__global__ void __launch_bounds__(kBlock) k_dfsph_divergence(Fluid<R> f, const P4<R>* __restrict__ bpos, GridView g,
                                                             const uint32_t* __restrict__ cs, const uint32_t* __restrict__ bs,
                                                             Consts<R> c, int akinci, DevScalars* sc, LoopLimits lim,
                                                             double* partials, cudaGraphConditionalHandle cond)
{
    __shared__ double sh[33];
    if (!INITIAL && !sc->active) return;
    const uint32_t t = gtid();
    const uint32_t i = t / G;
    const int lane = (int)(t % G);
    const bool valid = i < f.count();
    R dv = 0;
    unsigned nn = 0;
    V3<R> xi = {0, 0, 0};
    if (valid) {
        xi = xyz(f.pos[i]);
        const V3<R> vi = xyz(f.vel[i]);
        const uint32_t pc = f.cell[i];
        walk<R, G>(g, cs, pc, xi, c.h, lane, [&](uint32_t j, V3<R> s) {
            const V3<R> r = s - xyz(ldg4(f.pos + j));
            const R r2 = dot3(r, r);
            if (r2 <= c.cull2) {
                const V3<R> gr = cubic_gradW(c, r, r2);
                dv += c.mass * dot3(vi - xyz(ldg4(f.vel + j)), gr);
                if (dot3(gr, gr) > (R)0) nn++;
            }
        });
        if (akinci)
            walk<R, G>(g, bs, pc, xi, c.h, lane, [&](uint32_t j, V3<R> s) {
                const P4<R> pb = ldg4(bpos + j);
                const V3<R> r = s - xyz(pb);
                const R r2 = dot3(r, r);
                if (r2 <= c.cull2) dv += pb.w * dot3(vi, cubic_gradW(c, r, r2));
            });
    }
    if (G > 1) { dv = group_sum<G>(dv); nn = group_sum<G>(nn); }
    double err = 0.0;
    if (valid && lane == 0) {
        const R dt = (R)sc->dt;
        dv = nn < 20u ? (R)0 : (dv < (R)0 ? (R)0 : dv);
        f.div[i] = dv;
        const R kv = dv * f.alpha[i] / (dt * f.rho[i]);
        f.xk[i] = P4<R>{xi.x, xi.y, xi.z, kv};
        err = rel_error(c, (double)dv);
    }
    double total;
    if (finish_reduction<false>(err, partials, &sc->block_counter, sh, &total) && threadIdx.x == 0) {
        const double avg = total / (double)f.count();
        const double lim_v = lim.maxErrorV / sc->dt;
        if (!isfinite(avg)) sc->status |= ST_NONFINITE;
        if (INITIAL) {
            sc->iterationsV = 0;
            sc->avgDivError = avg;
            sc->active = (lim.minItV > 0u) && (lim.maxIt > 0u);
            if (!sc->active) sc->avgDivError = 0.0;
        } else {
            const unsigned it = ++sc->iterationsV;
            sc->avgDivError = avg;
            const unsigned act = ((avg > lim_v) || (it < lim.minItV)) && (it < lim.maxIt);
            sc->active = act;
            if (!act) {
                sc->sumIterationsV += it;
                if (it >= lim.maxIt && avg > lim_v) sc->status |= ST_ITER_CAP_V;
            }
        }
        if (cond) cudaGraphSetConditional(cond, sc->active);
    }
}

// ===========================================================================
// Integration and the cube boundary
// ===========================================================================

// CubeBoundaryModel::correctPositionAndVelocity CubeBoundaryModel.cpp:16-94
// with normalFct 0 and tangentialFct 1 (CubeBoundaryModel::init :5-14).
template <typename R>
__device__ __forceinline__ void cube_clamp(P4<R>& p, P4<R>& v, uint32_t cell, const GridView& g, double h, const Consts<R>& c)
{
    double a[3];
    abs_pos(p, cell, g, h, a);
    const R normalFct = 0, tangentialFct = 1;
    double mn[3] = {(double)c.cube_min[0], (double)c.cube_min[1], (double)c.cube_min[2]};
    double mx[3] = {(double)c.cube_max[0], (double)c.cube_max[1], (double)c.cube_max[2]};
    R* vv[3] = {&v.x, &v.y, &v.z};
    bool changed[3] = {false, false, false};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        R& vd = *vv[d];
        R& o1 = *vv[(d + 1) % 3];
        R& o2 = *vv[(d + 2) % 3];
        if (a[d] < mn[d]) {
            a[d] = mn[d]; changed[d] = true;
            if (vd < (R)0) vd *= -normalFct;
            o1 *= tangentialFct; o2 *= tangentialFct;
        } else if (a[d] > mx[d]) {
            a[d] = mx[d]; changed[d] = true;
            if (vd > (R)0) vd *= -normalFct;
            o1 *= tangentialFct; o2 *= tangentialFct;
        }
    }
    if constexpr (sizeof(R) == 4) {
        if (changed[0]) p.x = (R)(a[0] - (double)(cell_x(cell) + g.ox) * h);
        if (changed[1]) p.y = (R)(a[1] - (double)(cell_y(cell) + g.oy) * h);
        if (changed[2]) p.z = (R)(a[2] - (double)(cell_z(cell) + g.oz) * h);
    } else {
        p.x = a[0]; p.y = a[1]; p.z = a[2];
    }
}

template <typename R>
__global__ void k_dfsph_cube(Fluid<R> f, GridView g, double h, Consts<R> c)
{
    const uint32_t i = gtid();
    if (i >= f.count()) return;
    P4<R> p = f.pos[i], v = f.vel[i];
    cube_clamp(p, v, f.cell[i], g, h, c);
    f.pos[i] = p;
    f.vel[i] = v;
}

// SPHSolver::integrate SPHSolver.cpp:141-170 (PCISPH: PCISPHSolver::integrate
// PCISPHSolver.cpp:444-473 adds the pressure acceleration), then the cube
// boundary when present.
template <typename R, bool PCI>
__global__ void k_integrate(Fluid<R> f, GridView g, double h, Consts<R> c, const DevScalars* __restrict__ sc)
{
    const uint32_t i = gtid();
    if (i >= f.count()) return;
    const R dt = (R)sc->dt;
    P4<R> a = f.acc[i], v = f.vel[i], p = f.pos[i];
    if (PCI) {
        const P4<R> pa = f.pacc[i];
        a.x = a.x + (c.gx + pa.x); a.y = a.y + (c.gy + pa.y); a.z = a.z + (c.gz + pa.z);
    } else {
        a.x = a.x + c.gx; a.y = a.y + c.gy; a.z = a.z + c.gz;
    }
    v.x = v.x + a.x * dt; v.y = v.y + a.y * dt; v.z = v.z + a.z * dt;
    p.x = p.x + v.x * dt; p.y = p.y + v.y * dt; p.z = p.z + v.z * dt;
    if (c.has_cube) cube_clamp(p, v, f.cell[i], g, h, c);
    f.acc[i] = P4<R>{0, 0, 0, 0};
    f.vel[i] = v;
    f.pos[i] = p;
}

// ===========================================================================
// PCISPH (PCISPHSolver.cpp)
// ===========================================================================

// PCISPHSolver::initPressure PCISPHSolver.cpp:83-120
template <typename R>
__global__ void k_pcisph_init(Fluid<R> f)
{
    const uint32_t i = gtid();
    if (i >= f.count()) return;
    f.press[i] = 0;
    f.pacc[i] = P4<R>{0, 0, 0, 0};
}

// Loop entry of PCISPHSolver::pressureSolver PCISPHSolver.cpp:362-365: the
// previous step's maximum density error is tested, as the reference does.
static __global__ void k_pcisph_loop_begin(DevScalars* sc, LoopLimits lim, cudaGraphConditionalHandle cond)
{
    sc->iterations = 0;
    sc->disp_bits = 0u;
    sc->active = ((sc->maxDensityError > lim.maxError) || (0u < lim.minIt)) && (0u < lim.maxIt);
    if (cond) cudaGraphSetConditional(cond, sc->active);
}

// PCISPHSolver::predictVelocityAndPosition PCISPHSolver.cpp:122-149
// With TRACK, also the largest |predicted - current position| of the loop
// so far into sc->disp_bits (the candidate lists' validity).
template <typename R, bool TRACK = false>
__global__ void k_pcisph_predict(Fluid<R> f, Consts<R> c, DevScalars* __restrict__ sc)
{
    if (!sc->active) return;
    const uint32_t i = gtid();
    float d = 0.f;
    if (i < f.count()) {
        const R dt = (R)sc->dt;
        const P4<R> a = f.acc[i], pa = f.pacc[i], v = f.vel[i], x = f.pos[i];
        const V3<R> acc = {(a.x + pa.x) + c.gx, (a.y + pa.y) + c.gy, (a.z + pa.z) + c.gz};
        const P4<R> pv = {v.x + acc.x * dt, v.y + acc.y * dt, v.z + acc.z * dt, 0};
        f.predV[i] = pv;
        const P4<R> pr = {x.x + pv.x * dt, x.y + pv.y * dt, x.z + pv.z * dt, 0};
        f.predR[i] = pr;
        if (TRACK) {
            const V3<R> dd = {pr.x - x.x, pr.y - x.y, pr.z - x.z};
            d = (float)sqrt(dot3(dd, dd));
            if (!(d >= 0.f)) d = INFINITY;   // NaN: no list
        }
    }
    if (TRACK) {
        // block maximum, then one atomic per block (blockDim.x <= 1024)
        __shared__ float wmax[32];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) d = fmaxf(d, __shfl_down_sync(0xffffffffu, d, o));
        if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = d;
        __syncthreads();
        if (threadIdx.x == 0) {
            float m = 0.f;
            for (unsigned w = 0; w < (blockDim.x + 31) / 32; ++w) m = fmaxf(m, wmax[w]);
            if (m > 0.f) atomicMax(&sc->disp_bits, __float_as_uint(m));
        }
    }
}

// PCISPHSolver::predictFluidDensities PCISPHSolver.cpp:164-212 (predicted
// positions, cells of the current positions) fused with
// PCISPHSolver::updatePressure PCISPHSolver.cpp:249-295 (max reduction) and
// the p/rho^2 hand-off to the pressure-acceleration walk.
template <typename R, int G>
__global__ void __launch_bounds__(kBlock) k_pcisph_density_pressure(Fluid<R> f, const P4<R>* __restrict__ bpos, GridView g,
                                                                    const uint32_t* __restrict__ cs, const uint32_t* __restrict__ bs,
                                                                    Consts<R> c, int akinci, DevScalars* sc, LoopLimits lim,
                                                                    double* partials,
                                                                    CandLists L = CandLists{nullptr, nullptr, 0u},
                                                                    float margin = 0.f)
{
    __shared__ double sh[33];
    if (!sc->active) return;
    const uint32_t t = gtid();
    const uint32_t i = t / G;
    const int lane = (int)(t % G);
    const bool valid = i < f.count();
    // the lists hold every candidate that can come within h while each
    // predicted displacement stays below margin / 2 (10 % slack for rounding)
    if (L.idx && !(2.f * __uint_as_float(sc->disp_bits) <= 0.9f * margin)) L.idx = nullptr;
    R density = 0;
    if (valid) {
        const V3<R> xi = xyz(f.predR[i]);
        const uint32_t pc = f.cell[i];
        fluid_visit<R, G, false>(L, f.n, i, g, cs, pc, xi, c.h, lane, [&](uint32_t j, V3<R> s) {
            const V3<R> r = s - xyz(ldg4(f.predR + j));
            const R r2 = dot3(r, r);
            if (r2 <= c.cull2) density += c.mass * cubic_W(c, sqrt(r2));
        });
        if (akinci)
            walk<R, G>(g, bs, pc, xi, c.h, lane, [&](uint32_t j, V3<R> s) {
                const P4<R> pb = ldg4(bpos + j);
                const V3<R> r = s - xyz(pb);
                const R r2 = dot3(r, r);
                if (r2 <= c.cull2) density += pb.w * cubic_W(c, sqrt(r2));
            });
    }
    if (G > 1) density = group_sum<G>(density);
    double err = 0.0;
    if (valid && lane == 0) {
        f.rho[i] = density;
        f.vel[i].w = density;
        const R e = density - c.density0 > (R)0 ? density - c.density0 : (R)0;
        const R p = f.press[i] + (R)sc->scaling * e;
        f.press[i] = p;
        const P4<R> x = f.pos[i];
        f.xk[i] = P4<R>{x.x, x.y, x.z, p / (density * density)};
        err = (double)(e / c.density0);
    }
    double mx;
    if (finish_reduction<true>(err, partials, &sc->block_counter, sh, &mx) && threadIdx.x == 0) {
        mx = fmax(mx, 0.0);
        sc->maxDensityError = mx;
        if (!isfinite(mx)) sc->status |= ST_NONFINITE;
        const unsigned it = sc->iterations + 1;
        sc->next_active = ((mx > lim.maxError) || (it < lim.minIt)) && (it < lim.maxIt);
    }
}

// PCISPHSolver::computePressureAcc PCISPHSolver.cpp:297-358 (Spiky gradient,
// current positions; xk.w = p/rho^2)
template <typename R, int G>
__global__ void __launch_bounds__(kBlock) k_pcisph_pressure_acc(Fluid<R> f, const P4<R>* __restrict__ bpos, GridView g,
                                                                const uint32_t* __restrict__ cs, const uint32_t* __restrict__ bs,
                                                                Consts<R> c, int akinci, const DevScalars* __restrict__ sc,
                                                                const R* __restrict__ bdp,
                                                                CandLists L = CandLists{nullptr, nullptr, 0u})
{
    if (!sc->active) return;
    const uint32_t t = gtid();
    const uint32_t i = t / G;
    const int lane = (int)(t % G);
    const bool valid = i < f.count();
    V3<R> pacc = {0, 0, 0};
    if (valid) {
        const P4<R> pi = f.xk[i];
        const V3<R> xi = xyz(pi);
        const R dpi = pi.w;
        const uint32_t pc = f.cell[i];
        fluid_visit<R, G>(L, f.n, i, g, cs, pc, xi, c.h, lane, [&](uint32_t j, V3<R> s) {
            const P4<R> pj = ldg4(f.xk + j);
            const V3<R> r = s - xyz(pj);
            const R r2 = dot3(r, r);
            if (r2 <= c.cull2) pacc = pacc - (c.mass * (dpi + pj.w)) * spiky_gradW(c, r, r2);
        });
        if (akinci)
            walk<R, G>(g, bs, pc, xi, c.h, lane, [&](uint32_t j, V3<R> s) {
                const P4<R> pb = ldg4(bpos + j);
                const V3<R> r = s - xyz(pb);
                const R r2 = dot3(r, r);
                // PCISPHSolver.cpp:332-356, as the WCSPH force
                const R q = bdp ? dpi + bdp[j] : dpi;
                if (r2 <= c.cull2) pacc = pacc - (pb.w * q) * spiky_gradW(c, r, r2);
            });
    }
    if (G > 1) pacc = group_sum3<G>(pacc);
    if (!valid || lane != 0) return;
    f.pacc[i] = P4<R>{pacc.x, pacc.y, pacc.z, 0};
}

// ===========================================================================
// PCISPH boundary model (PCISPHBoundaryModel.cpp): boundary particles with
// the fluid's mass, normals, and their own densities and pressures.
// ===========================================================================

// SPHSolver::computeBoundaryDensities SPHSolver.cpp:94-127 (cubic spline,
// current positions; MODE 0), followed by WCSPHSolver::computeBoundaryPressures
// WCSPHSolver.cpp:97-114 (MODE 1); or PCISPHSolver::predictBoundaryDensities
// PCISPHSolver.cpp:214-247 (Poly6, predicted fluid positions) followed by the
// boundary part of updatePressure :276-293 (MODE 2, inside the loop).
// MODE 1 and 2 also store p / rho^2 for the pressure walks.
template <typename R, int MODE>
__global__ void k_bh_boundary(Boundary<R> b, Fluid<R> f, GridView g, const uint32_t* __restrict__ cs,
                              const uint32_t* __restrict__ bs, Consts<R> c, const DevScalars* __restrict__ sc)
{
    if (MODE == 2 && !sc->active) return;
    const uint32_t i = gtid();
    if (i >= b.n) return;
    const V3<R> xi = xyz(b.pos[i]);
    const uint32_t pc = b.cell[i];
    const P4<R>* fx = MODE == 2 ? f.predR : f.pos;
    R density = 0;
    // the fluid candidates' predicted positions (MODE 2) may lie outside the
    // cells they are filed by: no trimming then
    auto fluid_term = [&](uint32_t j, V3<R> s) {
        const V3<R> r = s - xyz(ldg4(fx + j));
        const R r2 = dot3(r, r);
        if (r2 <= c.cull2) density += c.mass * (MODE == 2 ? poly6_W(c, r2) : cubic_W(c, sqrt(r2)));
    };
    if (MODE == 2) walk<R, 1, false>(g, cs, pc, xi, c.h, 0, fluid_term);
    else walk<R, 1>(g, cs, pc, xi, c.h, 0, fluid_term);
    walk<R, 1>(g, bs, pc, xi, c.h, 0, [&](uint32_t j, V3<R> s) {
        const V3<R> r = s - xyz(ldg4(b.pos + j));
        const R r2 = dot3(r, r);
        if (r2 <= c.cull2) density += c.mass * (MODE == 2 ? poly6_W(c, r2) : cubic_W(c, sqrt(r2)));
    });
    b.dens[i] = density;
    if (MODE == 0) return;
    R p;
    if (MODE == 1) {
        p = fmax((R)0, c.k_eos * (pow(density / c.density0, c.gamma) - (R)1));
    } else {
        const R e = density - c.density0 > (R)0 ? density - c.density0 : (R)0;
        p = b.press[i] + (R)sc->scaling * e;
    }
    b.press[i] = p;
    b.dp[i] = p / (density * density);
}

// One more grid build (cell lifetimes of the PCISPH boundary model).
static __global__ void k_bh_epoch(DevScalars* sc) { sc->grid_epoch += 1; }

// Cells holding boundary points exist from the first build on.
static __global__ void k_bh_mark_cells(uint32_t n, const uint32_t* __restrict__ key, uint32_t* __restrict__ cell_epoch)
{
    const uint32_t i = gtid();
    if (i < n) atomicMin(cell_epoch + key[i], 1u);
}

// PCISPHSolver::initPressure PCISPHSolver.cpp:105-119: boundary pressures 0.
template <typename R>
__global__ void k_bh_zero_pressure(Boundary<R> b)
{
    const uint32_t i = gtid();
    if (i >= b.n) return;
    b.press[i] = 0;
    b.dp[i] = 0;
}

// PCISPHBoundaryModel::correctPositions :219-316 (MODE 0: weights from the
// current positions, WCSPH / DFSPH; MODE 1: from the predicted positions,
// PCISPH) and ::correctPredPositions :394-448 (MODE 2: corrects the
// predicted positions).  Boundary points closer than h/2 to the particle
// (current positions) push it back along the weighted mean of their normals;
// the particle's normal is always rewritten (normalised mean, NaN when no
// point is that close, as glm::normalize of a zero vector gives).  Cells
// must be current for the positions tested (positions rebased first).
template <typename R, int MODE>
__global__ void k_bh_collide(Fluid<R> f, Boundary<R> b, GridView g, const uint32_t* __restrict__ bs, Consts<R> c,
                             const DevScalars* __restrict__ sc, uint32_t* __restrict__ cell_epoch)
{
    if (MODE == 2 && !sc->active) return;
    const uint32_t i = gtid();
    if (i >= f.count()) return;
    const V3<R> xi = xyz(f.pos[i]);
    const uint32_t pc = f.cell[i];
    // The reference looks the candidates up in a hash table whose cells come
    // into existence when a point is inserted or a lookup creates them
    // (unordered_map::operator[]), and get candidate lists at the next
    // neighbour search: a particle in a cell that did not exist at the last
    // search (one that left the region ever occupied, or the grid box) has
    // no candidates, and the lookup creates the cell for the next search.
    bool has_cands = true;
    {
        bool out = false;
        if constexpr (sizeof(R) == 4) {
            out = !(xi.x >= (R)0 && xi.x < c.h && xi.y >= (R)0 && xi.y < c.h && xi.z >= (R)0 && xi.z < c.h);
        } else {
            out = (int)floor((double)xi.x / c.h) - g.ox != cell_x(pc) || (int)floor((double)xi.y / c.h) - g.oy != cell_y(pc) ||
                  (int)floor((double)xi.z / c.h) - g.oz != cell_z(pc);
        }
        if (out) {
            has_cands = false;
        } else if (cell_epoch) {
            const uint32_t k = cell_key(g, cell_x(pc), cell_y(pc), cell_z(pc));
            const unsigned E = sc->grid_epoch;
            if (cell_epoch[k] > E) {
                has_cands = false;
                atomicMin(cell_epoch + k, E + 1);
            }
        }
    }
    const V3<R> wi = MODE == 0 ? xi : xyz(f.predR[i]);
    const R rest = (R)0.5 * c.h;
    V3<R> avg = {0, 0, 0};
    R wsum = 0, w2sum = 0;
    if (has_cands) walk<R, 1>(g, bs, pc, xi, c.h, 0, [&](uint32_t j, V3<R> s) {
        const P4<R> pb = ldg4(b.pos + j);
        const V3<R> rib = s - xyz(pb);
        if (!(sqrt(dot3(rib, rib)) < rest)) return;
        V3<R> prib;
        if (MODE == 0) prib = rib;
        else if constexpr (sizeof(R) == 8) prib = wi - xyz(pb);
        else prib = rib + (wi - xi);  // the predicted position in the candidate's frame
        const R lp = sqrt(dot3(prib, prib));
        const R w = fmax((R)0, (rest - lp) / rest);
        wsum += w;
        w2sum += w * (rest - lp);
        avg = avg + w * xyz(ldg4(b.nrm + j));
    });
    const V3<R> ni = avg * ((R)1 / sqrt(dot3(avg, avg)));
    f.normal[i] = P4<R>{ni.x, ni.y, ni.z, 0};
    if (wsum > (R)0) {
        const V3<R> d = ((R)1 / wsum * w2sum) * ni;
        P4<R>* tgt = MODE == 2 ? f.predR : f.pos;
        P4<R> p = tgt[i];
        p.x = p.x + d.x; p.y = p.y + d.y; p.z = p.z + d.z;
        tgt[i] = p;
    }
}

// PCISPHBoundaryModel::correctVelocities :318-392: for particles with a valid
// normal, v = tangentialFct * v_t - normalFct * v_n of the velocity (PRED:
// of the last predicted velocity, PCISPH).
template <typename R, bool PRED>
__global__ void k_bh_correct_velocities(Fluid<R> f, Consts<R> c)
{
    const uint32_t i = gtid();
    if (i >= f.count()) return;
    const V3<R> ni = xyz(f.normal[i]);
    if (!(sqrt(dot3(ni, ni)) > (R)0)) return;
    const V3<R> u = xyz(PRED ? f.predV[i] : f.vel[i]);
    const V3<R> nVel = dot3(u, ni) * ni;
    const V3<R> tVel = u - nVel;
    const V3<R> v = c.bh_tf * tVel - c.bh_nf * nVel;
    P4<R> o = f.vel[i];
    o.x = v.x; o.y = v.y; o.z = v.z;
    f.vel[i] = o;
}

// Boundary normals from the host (FP64 xyz) and the model's mass as the
// walks' boundary weight.
template <typename R>
__global__ void k_bh_upload(const double* __restrict__ nrm, uint32_t n, Boundary<R> b, R mass)
{
    const uint32_t i = gtid();
    if (i >= n) return;
    b.nrm[i] = P4<R>{(R)nrm[3 * i], (R)nrm[3 * i + 1], (R)nrm[3 * i + 2], 0};
    b.pos[i].w = mass;
}

// End of one PCISPH iteration: PCISPHSolver.cpp:383 (++iterations) and the
// loop test for the next one.
static __global__ void k_pcisph_loop_next(DevScalars* sc, LoopLimits lim, cudaGraphConditionalHandle cond)
{
    if (!sc->active) return;
    const unsigned it = ++sc->iterations;
    sc->active = sc->next_active;
    if (!sc->active) {
        sc->sumIterations += it;
        if (it >= lim.maxIt && sc->maxDensityError > lim.maxError) sc->status |= ST_ITER_CAP;
    }
    if (cond) cudaGraphSetConditional(cond, sc->active);
}

// Pair-list occupancy for the statistics: stored pairs and overflowing particles.
static __global__ void k_list_stats(uint32_t n, const uint32_t* __restrict__ count, uint32_t kmax,
                                    unsigned long long* out)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t c = count[i];
    atomicAdd(out, (unsigned long long)(c < kmax ? c : kmax));
    if (c > kmax) atomicAdd(out + 1, 1ull);
}

// ===========================================================================
// Emitters (Emitter.cpp:85-161, FluidModel::emitParticles FluidModel.cpp:
// 145-149): particle groups appended at the end of the active slots.
// ===========================================================================
constexpr int kMaxEmitters = 64;

struct EmitterDev {
    double r[3];           // emitter position
    double v;              // emission speed along the emitter's local z
    double q[4];           // rotation quaternion (w, x, y, z)
    double next;           // nextTimeEmit
    double period;         // spacing * 1.105 * 2r / v, added after each emission
    uint32_t remaining;    // particles left to emit
    uint32_t first, count; // the group's points in the group table
    uint32_t pause;
};

// a x b, component order and operand order of GLM's cross().
__device__ __forceinline__ void cross_rn(const double a[3], const double b[3], double o[3])
{
    o[0] = __dsub_rn(__dmul_rn(a[1], b[2]), __dmul_rn(b[1], a[2]));
    o[1] = __dsub_rn(__dmul_rn(a[2], b[0]), __dmul_rn(b[2], a[0]));
    o[2] = __dsub_rn(__dmul_rn(a[0], b[1]), __dmul_rn(b[0], a[1]));
}

// Rotation of v by the unit quaternion q = (w, u): v + 2 (w (u x v) + u x (u x v)),
// GLM's quat * vec3, each operation rounded on its own.
__device__ __forceinline__ void quat_rotate_rn(const double q[4], const double v[3], double o[3])
{
    const double u[3] = {q[1], q[2], q[3]};
    double uv[3], uuv[3];
    cross_rn(u, v, uv);
    cross_rn(u, uv, uuv);
#pragma unroll
    for (int k = 0; k < 3; ++k) o[k] = __dadd_rn(v[k], __dmul_rn(__dadd_rn(__dmul_rn(uv[k], q[0]), uuv[k]), 2.0));
}

enum EmitFlags : unsigned { EMIT_PCISPH = 1u, EMIT_NORMALS = 2u };

// Simulation::emitParticles at the current time: thread 0 decides, in
// emitter order, which emitters fire (time >= nextTimeEmit, not paused, a
// whole group left: Emitter.cpp:85-97,105) and reserves their slots; then
// every particle of a firing group gets
//   x = R (g_i + t_off (v_e + gravity t_off)) + r,  v = R v_e,  v_e = (0, 0, v),
// t_off = time - nextTimeEmit (Emitter.cpp:107-124), in FP64.  One block.
template <typename R>
__global__ void __launch_bounds__(256) k_emit(Fluid<R> f, EmitterDev* __restrict__ em, int nem, const double* __restrict__ group,
                                              GridView g, double h, double gx, double gy, double gz, DevScalars* sc,
                                              uint32_t* __restrict__ na, unsigned flags)
{
    __shared__ uint32_t base[kMaxEmitters];
    __shared__ double toff[kMaxEmitters];
    __shared__ int any;
    if (threadIdx.x == 0) {
        uint32_t n = *na;
        const double t = sc->time;
        any = 0;
        for (int e = 0; e < nem; ++e) {
            EmitterDev& E = em[e];
            base[e] = 0xffffffffu;
            if (t >= E.next && !E.pause && E.count <= E.remaining) {
                base[e] = n;
                toff[e] = __dsub_rn(t, E.next);
                n += E.count;
                E.remaining -= E.count;
                E.next = __dadd_rn(E.next, E.period);
                any = 1;
            }
        }
        *na = n;
    }
    __syncthreads();
    if (!any) return;
    for (int e = 0; e < nem; ++e) {
        if (base[e] == 0xffffffffu) continue;
        const double to = toff[e];
        const EmitterDev& E = em[e];
        const double s[3] = {__dadd_rn(0.0, __dmul_rn(gx, to)), __dadd_rn(0.0, __dmul_rn(gy, to)), __dadd_rn(E.v, __dmul_rn(gz, to))};
        const double v0[3] = {0.0, 0.0, E.v};
        double vr[3];
        quat_rotate_rn(E.q, v0, vr);
        for (uint32_t k = threadIdx.x; k < E.count; k += blockDim.x) {
            const double* gp = group + 3 * (size_t)(E.first + k);
            const double p[3] = {__dadd_rn(gp[0], __dmul_rn(to, s[0])), __dadd_rn(gp[1], __dmul_rn(to, s[1])),
                                 __dadd_rn(gp[2], __dmul_rn(to, s[2]))};
            double pr[3];
            quat_rotate_rn(E.q, p, pr);
            const uint32_t i = base[e] + k;
            store_particle(f, i, __dadd_rn(pr[0], E.r[0]), __dadd_rn(pr[1], E.r[1]), __dadd_rn(pr[2], E.r[2]), vr[0], vr[1],
                           vr[2], g, h, sc);
            f.rho[i] = 0;
            f.alpha[i] = 0;
            f.div[i] = 0;
            f.pred[i] = 0;
            if (flags & EMIT_PCISPH) {
                f.predR[i] = P4<R>{0, 0, 0, 0};
                f.predV[i] = P4<R>{0, 0, 0, 0};
                f.pacc[i] = P4<R>{0, 0, 0, 0};
            }
            if (flags & EMIT_NORMALS) f.normal[i] = P4<R>{0, 0, 0, 0};
        }
    }
}

// Emitter::setPause (Emitter.cpp:80-84) on every emitter: the flag, and the
// next emission at the current time.
static __global__ void k_emit_pause(EmitterDev* __restrict__ em, int nem, uint32_t pause, const DevScalars* __restrict__ sc)
{
    const int e = (int)threadIdx.x;
    if (e < nem) {
        em[e].pause = pause;
        em[e].next = sc->time;
    }
}

// Simulation::step bookkeeping: time += dt, steps++ (DFSPHSolver.cpp:111).
static __global__ void k_finish_step(DevScalars* sc)
{
    sc->time = sc->time + sc->dt;
    sc->steps += 1;
}

// ===========================================================================
// Neighbour sets for the parity tests: candidates of the particle's cell
// within the cubic spline's support (q = |xi - xj| / h <= 1,
// CubicSpline.h:31), listed in walk order, indexed by original id.
// ===========================================================================
template <typename R>
__global__ void k_neighbors(Fluid<R> f, const P4<R>* __restrict__ bpos, const uint32_t* __restrict__ bid,
                            const uint32_t* __restrict__ bcell, GridView g,
                            const uint32_t* __restrict__ cs, const uint32_t* __restrict__ bs, Consts<R> c, double hd,
                            const int* __restrict__ off, const int* __restrict__ boff, int* __restrict__ cnt,
                            int* __restrict__ bcnt, int* __restrict__ nbr, int* __restrict__ bnbr, int* __restrict__ cells,
                            int* __restrict__ rank)
{
    const uint32_t i = gtid();
    if (i >= f.count()) return;
    const uint32_t me = f.id[i];
    const uint32_t pc = f.cell[i];
    double xi[3];
    abs_pos(f.pos[i], pc, g, hd, xi);
    int nf = 0, nb = 0;
    const int o = off ? off[me] : 0, bo = boff ? boff[me] : 0;
    walk<R, 1>(g, cs, pc, xyz(f.pos[i]), c.h, 0, [&](uint32_t j, V3<R>) {
        double xj[3];
        abs_pos(f.pos[j], f.cell[j], g, hd, xj);
        const double rx = xi[0] - xj[0], ry = xi[1] - xj[1], rz = xi[2] - xj[2];
        if (sqrt(rx * rx + ry * ry + rz * rz) / hd <= 1.0) {
            if (nbr) nbr[o + nf] = (int)f.id[j];
            nf++;
        }
    });
    walk<R, 1>(g, bs, pc, xyz(f.pos[i]), c.h, 0, [&](uint32_t j, V3<R>) {
        double xj[3];
        abs_pos(bpos[j], bcell[j], g, hd, xj);
        const double rx = xi[0] - xj[0], ry = xi[1] - xj[1], rz = xi[2] - xj[2];
        if (sqrt(rx * rx + ry * ry + rz * rz) / hd <= 1.0) {
            if (bnbr) bnbr[bo + nb] = (int)bid[j];
            nb++;
        }
    });
    if (cnt) cnt[me] = nf;
    if (bcnt) bcnt[me] = nb;
    if (cells) {
        cells[3 * me] = cell_x(pc) + g.ox; cells[3 * me + 1] = cell_y(pc) + g.oy; cells[3 * me + 2] = cell_z(pc) + g.oz;
    }
    if (rank) {
        const uint32_t k = cell_key(g, cell_x(pc), cell_y(pc), cell_z(pc));
        rank[me] = (int)(i - cs[k]);
    }
}

}  // namespace sph
