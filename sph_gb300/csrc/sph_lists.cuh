// Pair lists for the DFSPH solves.
//
// Between two grid builds the DFSPH step never moves a particle: the
// divergence solve, the next step's warm start and its density solve all run
// at the positions of the last build (DFSPHSolver.cpp:63-97).  So right after
// each build one 27-cell walk computes the densities and alpha factors
// (SPHSolver.cpp:44-91, DFSPHSolver.cpp:114-189) and records, per particle,
// every fluid neighbour with a non-zero kernel gradient together with
// m * gradW_ij, plus the summed Akinci boundary gradient
// sum_b rho0 psi_b gradW_ib.  The solver walks then read those lists instead
// of rescanning ~216 candidates and re-evaluating the kernel per pair.
//
// Layout: slot-major, pairs[k * n + i] = {m gradW_ij, as_float(j)}, so the
// threads of a warp (consecutive particles) read one contiguous 16-byte line
// per slot.  A particle with more than kmax neighbours keeps its count and
// falls back to the cell walk in every list kernel.
//
// Neighbours are listed in the cell walk's order, so each fluid sum adds the
// same non-zero terms in the same order as the reference; the boundary sum is
// pre-added once per build (a re-association of the reference's boundary
// terms, which all share the factor of particle i).
#pragma once

#include <cuda_fp16.h>

#include <cstring>
#include <vector>

#include "sph_kernels.cuh"

namespace sph {

template <typename R> struct Lists {
    P4<R>* pairs;       // kmax * n, slot-major: {m gradW_ij, as-bits j}
    uint32_t* count;    // neighbours with a non-zero gradient (may exceed kmax)
    P4<R>* bgrad;       // xyz: sum_b rho0 psi_b gradW_ib
    R* kbuf;            // k (or kv) of the pass in progress
    uint32_t kmax;
    // FP32 form: a half-precision copy of the cell-relative positions for
    // the build's cull, two particles per 16-byte word ({x, y, z, unused}
    // half2 pairs, z in the cell's modulo-3 frame), or nullptr
    const uint4* posh;
    unsigned* fault;    // status word of the bounds-checked build (SPH_INDEX_OK)
    // Akinci boundary points in the same half-precision form (static between
    // re-layouts) and their cells, for the boundary cull; or nullptr
    const uint4* bposh;
    const uint32_t* bcell;
};

// Phase 1 of the FP32 list build from the half-precision positions: the
// nine columns of the 27-cell neighbourhood (trimmed as walk() trims them),
// two candidates per half2 operation, accepted indices queued in walk order.
// The caller guarantees that the particle's cell is at least two cells from
// every face of the grid box (all 27 cells exist and hold in-grid particles,
// offsets in [0, h)) and that its own offsets are inside [-h/2, 3h/2].
//
// z needs no per-candidate cell: positions carry z in the frame of their
// cell's z index modulo 3 (in [0, 3h)), so for a candidate in cells
// z-1..z+1 the difference d of the two frame values is the true z distance
// plus a multiple of 3h, and min(|d|, 3h - |d|) is the true |dz| whenever
// |dz| <= 1.5h and above h (so culled) otherwise, up to a sliver of
// |dz| in [1.97h, 2h) that phase 2 drops.
//
// The test uses r^2 <= 1.03 h^2: for a pair within h, half-precision values
// (relative error 2^-11 each; x, y operands within 2.5h, z within 3h)
// move r^2 by less than 1.7 % of h^2, so every pair the FP32 test accepts
// is kept; pairs beyond h evaluate to W = 0, grad W = 0 in phase 2 and are
// dropped there.  Returns the number of accepted candidates (the queue
// holds the first qcap).
__device__ __forceinline__ __half2 as_half2(uint32_t u) { return *reinterpret_cast<const __half2*>(&u); }

__device__ __forceinline__ uint32_t cull_half(const GridView& g, const uint32_t* __restrict__ starts, uint32_t pc,
                                              V3<float> xi, float h, float cull2, const uint4* __restrict__ posh,
                                              uint32_t* q, uint32_t qstride, uint32_t qcap)
{
    const int cx = cell_x(pc), cy = cell_y(pc), cz = cell_z(pc);
    const float ofx = xi.x, ofy = xi.y, ofz = xi.z;
    const float gxm = ofx > 0.f ? ofx * ofx : 0.f, gxp = h - ofx > 0.f ? (h - ofx) * (h - ofx) : 0.f;
    const float gym = ofy > 0.f ? ofy * ofy : 0.f, gyp = h - ofy > 0.f ? (h - ofy) * (h - ofy) : 0.f;
    const float gzm = ofz > 0.f ? ofz * ofz : 0.f, gzp = h - ofz > 0.f ? (h - ofz) * (h - ofz) : 0.f;
    const float lim = h * h * (float)(1.0 + 1e-5);
    const __half2 thr = __float2half2_rn(cull2 * 1.03f);
    const __half2 zq = __float2half2_rn(zframe3(xi.z, cz, h));
    const __half2 h3 = __float2half2_rn(3.f * h);
    uint32_t nq = 0;
    // a column's candidate range (empty when trimmed); loaded one column ahead
    auto range = [&](int c, uint32_t* b, uint32_t* e) {
        const int dx = c / 3 - 1, dy = c - (c / 3) * 3 - 1;
        const float gxy = (dx < 0 ? gxm : (dx > 0 ? gxp : 0.f)) + (dy < 0 ? gym : (dy > 0 ? gyp : 0.f));
        if (!(gxy <= lim)) { *b = 0u; *e = 0u; return; }
        const uint32_t base = (__ldg(g.mortx + cx + dx) | __ldg(g.morty + cy + dy)) * (uint32_t)g.nz;
        *b = __ldg(starts + base + (gxy + gzm <= lim ? cz - 1 : cz));
        *e = __ldg(starts + base + (gxy + gzp <= lim ? cz + 2 : cz + 1));
    };
    uint32_t nb, ne;
    range(0, &nb, &ne);
#pragma unroll 1
    for (int c = 0; c < 9; ++c) {
        const int dx = c / 3 - 1, dy = c - (c / 3) * 3 - 1;
        const uint32_t bb = nb, ee = ne;
        if (c < 8) range(c + 1, &nb, &ne);
        const __half2 sx = __float2half2_rn(xi.x - (float)dx * h), sy = __float2half2_rn(xi.y - (float)dy * h);
        // The column's candidates 32 at a time (16 words): the test's
        // acceptance bits are gathered into one word, candidate j0 + b at
        // bit b, and only the accepted candidates (about one in five) are
        // queued, in walk order.
        for (uint32_t j0 = bb & ~1u; j0 < ee; j0 += 32) {
            const uint32_t nw = min(16u, (ee - j0 + 1) >> 1);
            const uint4* __restrict__ wp = posh + (j0 >> 1);
            // acceptance mask of one word: 0xffff per accepted half
            auto test = [&](const uint4 w) {
                const __half2 ddx = __hsub2(sx, as_half2(w.x));
                const __half2 ddy = __hsub2(sy, as_half2(w.y));
                const __half2 dz = __habs2(__hsub2(zq, as_half2(w.z)));
                const __half2 ddz = __hmin2(dz, __hsub2(h3, dz));
                const __half2 r2 = __hfma2(ddz, ddz, __hfma2(ddy, ddy, __hmul2(ddx, ddx)));
                return __hle2_mask(r2, thr);
            };
            // Two words (four candidates) per iteration: bytes 0 and 2 of
            // each mask (one per half) gathered into one word, then bit 8k+k
            // of that word's byte k moved to bit 24+k by one multiply (the
            // shifted copies land on distinct bits, so nothing carries).  An
            // odd word count reads one word past the range (the buffer holds
            // a spare word); its bits are cleared below.
            uint32_t bits = 0;
#pragma unroll 1
            for (uint32_t k = 0; k < nw; k += 2) {
                const unsigned m0 = test(__ldg(wp + k)), m1 = test(__ldg(wp + k + 1));
                const uint32_t u = __byte_perm(m0, m1, 0x6420u) & 0x08040201u;
                bits |= ((u * 0x01010101u) >> 24) << (2 * k);
            }
            if (nw < 16u) bits &= (1u << (2 * nw)) - 1u;
            // the first word's low particle may precede the column's range
            // (bb odd), the last word's high one follow it (ee odd)
            if (j0 < bb) bits &= ~1u;
            if (j0 + 2 * nw > ee) bits &= ~(1u << (2 * nw - 1));
            while (bits) {
                const uint32_t b = __ffs(bits) - 1;
                bits &= bits - 1;
                if (nq < qcap) q[nq * qstride + threadIdx.x] = j0 + b;
                ++nq;
            }
        }
    }
    return nq;
}

__device__ __forceinline__ float idx_as(float, uint32_t j) { return __uint_as_float(j); }
__device__ __forceinline__ double idx_as(double, uint32_t j) { return __longlong_as_double((long long)j); }
__device__ __forceinline__ uint32_t as_idx(float w) { return __float_as_uint(w); }
__device__ __forceinline__ uint32_t as_idx(double w) { return (uint32_t)__double_as_longlong(w); }

// Densities + alpha + the lists, one thread per particle, in two phases:
// the cell walk only culls candidates (distance test) and queues the
// accepted indices in shared memory; the kernel values are then evaluated in
// a dense loop over the queue.  (Evaluating inside the walk makes each warp
// execute the expensive branch on nearly every candidate, since some lane
// almost always accepts.)  A particle whose queue overflows is evaluated
// inside the walk instead.
constexpr uint32_t kQueue = 64;

template <typename R>
__device__ __forceinline__ V3<R> pair_vec(V3<R> xi, uint32_t ci, const P4<R>& pj, uint32_t cj, R h)
{
    if constexpr (sizeof(R) == 4) {
        const V3<R> s = {xi.x - (R)(cell_x(cj) - cell_x(ci)) * h, xi.y - (R)(cell_y(cj) - cell_y(ci)) * h,
                         xi.z - (R)(cell_z(cj) - cell_z(ci)) * h};
        return s - xyz(pj);
    } else {
        return xi - xyz(pj);
    }
}

// Per-particle body shared by the single-scene and the pool kernels; q is
// the block's shared queue (kQueue x kBlock).
template <typename R> struct BuildSums {
    R density, sumSq;
    V3<R> sumGrad;
    uint32_t cnt;
};

// Particles whose candidates overflow the shared queue: the whole
// evaluation inside the walk.  Out of line, so the common path's register
// allocation does not carry it.
template <typename R, bool FAST>
__device__ __noinline__ BuildSums<R> build_walk_all(uint32_t i, const Fluid<R>& f, const GridView& g,
                                                    const uint32_t* __restrict__ cs, const Consts<R>& c, const Lists<R>& L,
                                                    V3<R> xi, uint32_t pc)
{
    const uint32_t n = f.n;
    BuildSums<R> b{0, 0, {0, 0, 0}, 0};
    walk<R, 1>(g, cs, pc, xi, c.h, 0, [&](uint32_t j, V3<R> s) {
        const V3<R> r = s - xyz(ldg4(f.pos + j));
        const R r2 = dot3(r, r);
        if (!(r2 <= c.cull2)) return;
        R w;
        V3<R> gw;
        cubic_W_gradW<FAST>(c, r, r2, &w, &gw);
        b.density += c.mass * w;
        const V3<R> mg = c.mass * gw;
        const R mg2 = dot3(mg, mg);
        if (mg2 > (R)0) {
            b.sumGrad = b.sumGrad + mg;
            if constexpr (sizeof(R) == 8) {
                const R m = sqrt(mg2);
                b.sumSq += m * m;
            } else {
                b.sumSq += mg2;
            }
            if (b.cnt < L.kmax) L.pairs[(size_t)b.cnt * n + i] = P4<R>{mg.x, mg.y, mg.z, idx_as(R(0), j)};
            ++b.cnt;
        }
    });
    return b;
}

// Forward declarations: the list build's DIV0 form ends with the velocity
// divergence the first divergence-error pass would compute from the lists.
template <typename R> struct DivSum;
template <typename R>
__device__ __noinline__ DivSum<R> velocity_div_cells(const Fluid<R>& f, const P4<R>* __restrict__ bpos, const GridView& g,
                                                     const uint32_t* __restrict__ cs, const uint32_t* __restrict__ bs,
                                                     const Consts<R>& c, int akinci, uint32_t i, V3<R> vi);

template <typename R>
__device__ __noinline__ R reread_div(const Fluid<R>& f, const Lists<R>& L, uint32_t i, V3<R> vi, uint32_t cnt)
{
    const uint32_t n = f.n;
    R dv = 0;
    for (uint32_t k = 0; k < cnt; ++k) {
        const P4<R> pr = L.pairs[(size_t)k * n + i];
        const uint32_t j = as_idx(pr.w);
        if (!SPH_INDEX_OK(j, n, L.fault)) continue;
        dv += dot3(vi - xyz(f.vel[j]), xyz(pr));
    }
    return dv;
}

// DIV0: also sum m (v_i - v_j) . gradW_ij over the pairs as they are listed,
// plus v_i . (boundary gradient): the value velocity_div_one would read from
// the finished lists (same terms, same order), into *div0, with the count of
// neighbours into *nn0 (a particle whose list or queue overflowed takes the
// same list or cell walk as velocity_div_one).
template <typename R, bool FAST = false, bool DIV0 = false>
__device__ __forceinline__ void build_lists_one(uint32_t i, const Fluid<R>& f, const P4<R>* __restrict__ bpos,
                                                const GridView& g, const uint32_t* __restrict__ cs,
                                                const uint32_t* __restrict__ bs, const Consts<R>& c, int akinci,
                                                const Lists<R>& L, uint32_t* q, uint32_t qstride = kBlock,
                                                uint32_t qdepth = kQueue, R* div0 = nullptr, uint32_t* nn0 = nullptr)
{
    const uint32_t n = f.n;
    const V3<R> xi = xyz(f.pos[i]);
    const uint32_t pc = f.cell[i];
    const uint32_t qcap = L.kmax < qdepth ? L.kmax : qdepth;
    R density = 0, sumSq = 0;
    V3<R> sumGrad = {0, 0, 0};
    uint32_t cnt = 0;
    V3<R> vi = {0, 0, 0};
    if constexpr (DIV0) vi = xyz(f.vel[i]);
    R dv = 0;
    // vj: the neighbour's velocity (DIV0), loaded beside its position
    auto accept = [&](uint32_t j, V3<R> r, R r2, V3<R> vj) {
        R w;
        V3<R> gw;
        cubic_W_gradW<FAST>(c, r, r2, &w, &gw);
        density += c.mass * w;
        const V3<R> mg = c.mass * gw;
        const R mg2 = dot3(mg, mg);
        if (mg2 > (R)0) {
            sumGrad = sumGrad + mg;
            if constexpr (sizeof(R) == 8) {
                const R m = sqrt(mg2);
                sumSq += m * m;
            } else {
                sumSq += mg2;
            }
            if (cnt < L.kmax) L.pairs[(size_t)cnt * n + i] = P4<R>{mg.x, mg.y, mg.z, idx_as(R(0), j)};
            ++cnt;
            if constexpr (DIV0) dv += dot3(vi - vj, mg);
        }
    };
    // phase 1: cull.  The half-precision cull needs all 27 cells inside the
    // grid box and clear of its border cells (where particles that left the
    // box are kept, with unbounded offsets), and in-cell offsets; elsewhere
    // the cull runs in FP32.
    uint32_t nq = 0;
    bool half_cull = false;
    if constexpr (FAST && sizeof(R) == 4) {
        const R hh = (R)0.5 * c.h;
        const int cx = cell_x(pc), cy = cell_y(pc), cz = cell_z(pc);
        half_cull = L.posh && cx >= 2 && cy >= 2 && cz >= 2 && cx <= g.nx - 3 && cy <= g.ny - 3 && cz <= g.nz - 3 &&
                    fabsf(xi.x - hh) <= c.h && fabsf(xi.y - hh) <= c.h && fabsf(xi.z - hh) <= c.h;
        if (half_cull) nq = cull_half(g, cs, pc, xi, c.h, c.cull2, L.posh, q, qstride, qcap);
    }
    if (!half_cull)
        walk<R, 1, true, FAST>(g, cs, pc, xi, c.h, 0, [&](uint32_t j, V3<R> s) {
            const V3<R> r = s - xyz(ldg4(f.pos + j));
            if (dot3(r, r) <= c.cull2) {
                if (nq < qcap) q[nq * qstride + threadIdx.x] = j;
                ++nq;
            }
        });
    if (nq <= qcap) {
        // phase 2: evaluate the queued candidates in walk order
        for (uint32_t k = 0; k < nq; ++k) {
            const uint32_t j = q[k * qstride + threadIdx.x];
            // (a plain load for the velocity: other threads write its w here)
            V3<R> vj = {0, 0, 0};
            if constexpr (DIV0) vj = xyz(f.vel[j]);
            const V3<R> r = pair_vec(xi, pc, ldg4(f.pos + j), __ldg(f.cell + j), c.h);
            accept(j, r, dot3(r, r), vj);
        }
    } else {
        const BuildSums<R> b = build_walk_all<R, FAST>(i, f, g, cs, c, L, xi, pc);
        density = b.density;
        sumSq = b.sumSq;
        sumGrad = b.sumGrad;
        cnt = b.cnt;
    }
    V3<R> bg = {0, 0, 0};
    if (akinci) {
        auto bterm = [&](const P4<R>& pb, V3<R> r) {
            const R r2 = dot3(r, r);
            if (!(r2 <= c.cull2)) return;
            R w;
            V3<R> gw;
            cubic_W_gradW<FAST>(c, r, r2, &w, &gw);
            density += pb.w * w;
            bg = bg + pb.w * gw;
        };
        // The boundary candidates as the fluid ones: culled from the static
        // half-precision copy into the (now free) queue, then evaluated in
        // the walk's order (the same cells, trimmed alike: the same terms in
        // the same order as the walk, the gradient sum compiled apart from
        // the walk's, so its last bit may differ); or the walk itself.
        uint32_t nb = qcap + 1u;
        if constexpr (FAST && sizeof(R) == 4) {
            if (half_cull && L.bposh) nb = cull_half(g, bs, pc, xi, c.h, c.cull2, L.bposh, q, qstride, qcap);
        }
        if (nb <= qcap) {
            for (uint32_t k = 0; k < nb; ++k) {
                const uint32_t j = q[k * qstride + threadIdx.x];
                const P4<R> pb = ldg4(bpos + j);
                bterm(pb, pair_vec(xi, pc, pb, __ldg(L.bcell + j), c.h));
            }
        } else {
            walk<R, 1>(g, bs, pc, xi, c.h, 0, [&](uint32_t j, V3<R> s) {
                const P4<R> pb = ldg4(bpos + j);
                bterm(pb, s - xyz(pb));
            });
        }
    }
    sumGrad = sumGrad + bg;
    f.rho[i] = density;
    f.vel[i].w = density;
    R den;
    if constexpr (sizeof(R) == 8) {
        const R m = sqrt(dot3(sumGrad, sumGrad));
        den = m * m + sumSq;
    } else {
        den = dot3(sumGrad, sumGrad) + sumSq;
    }
    f.alpha[i] = (fabs(den) > c.eps) ? density / den : (R)0;
    L.count[i] = cnt;
    L.bgrad[i] = P4<R>{bg.x, bg.y, bg.z, 0};
    if constexpr (DIV0) {
        if (cnt > L.kmax) {
            const DivSum<R> d = velocity_div_cells(f, bpos, g, cs, bs, c, akinci, i, vi);
            *div0 = d.dv;
            *nn0 = d.nn;
        } else {
            if (nq > qcap) dv = reread_div<R>(f, L, i, vi, cnt);
            if (akinci) dv += dot3(vi, bg);
            *div0 = dv;
            *nn0 = cnt;
        }
    }
}

template <typename R>
__global__ void __launch_bounds__(kBlock, 7) k_build_lists(Fluid<R> f, const P4<R>* __restrict__ bpos, GridView g,
                                                           const uint32_t* __restrict__ cs, const uint32_t* __restrict__ bs,
                                                           Consts<R> c, int akinci, Lists<R> L)
{
    __shared__ uint32_t q[kQueue * kBlock];
    const uint32_t i = gtid();
    if (i >= f.count()) return;
    build_lists_one<R, sizeof(R) == 4>(i, f, bpos, g, cs, bs, c, akinci, L, q);
}

// ---- cell-walk fallbacks for particles whose list overflowed -------------

template <typename R, int MODE>
__device__ __noinline__ V3<R> correct_sum_cells(const Fluid<R>& f, const P4<R>* __restrict__ bpos, const GridView& g,
                                   const uint32_t* __restrict__ cs, const uint32_t* __restrict__ bs, const Consts<R>& c,
                                   int akinci, uint32_t i, R ki, const R* __restrict__ kbuf)
{
    V3<R> sum = {0, 0, 0};
    const V3<R> xi = xyz(f.pos[i]);
    const uint32_t pc = f.cell[i];
    walk<R, 1>(g, cs, pc, xi, c.h, 0, [&](uint32_t j, V3<R> s) {
        const R kSum = ki + kbuf[j];
        if (!(fabs(kSum) > c.eps)) return;
        const V3<R> r = s - xyz(ldg4(f.pos + j));
        const R r2 = dot3(r, r);
        if (r2 <= c.cull2) sum = sum + (c.mass * kSum) * cubic_gradW(c, r, r2);
    });
    const R kb = MODE == 0 ? c.bwarm * ki : ki;
    if (akinci && fabs(kb) > c.eps)
        walk<R, 1>(g, bs, pc, xi, c.h, 0, [&](uint32_t j, V3<R> s) {
            const P4<R> pb = ldg4(bpos + j);
            const V3<R> r = s - xyz(pb);
            const R r2 = dot3(r, r);
            if (r2 <= c.cull2) sum = sum + (pb.w * kb) * cubic_gradW(c, r, r2);
        });
    return sum;
}

template <typename R> struct DivSum {
    R dv;
    uint32_t nn;
};

template <typename R>
__device__ __noinline__ DivSum<R> velocity_div_cells(const Fluid<R>& f, const P4<R>* __restrict__ bpos, const GridView& g,
                                                     const uint32_t* __restrict__ cs, const uint32_t* __restrict__ bs,
                                                     const Consts<R>& c, int akinci, uint32_t i, V3<R> vi)
{
    R dv = 0;
    unsigned cnt = 0;
    const V3<R> xi = xyz(f.pos[i]);
    const uint32_t pc = f.cell[i];
    walk<R, 1>(g, cs, pc, xi, c.h, 0, [&](uint32_t j, V3<R> s) {
        const V3<R> r = s - xyz(ldg4(f.pos + j));
        const R r2 = dot3(r, r);
        if (r2 <= c.cull2) {
            const V3<R> gr = cubic_gradW(c, r, r2);
            dv += c.mass * dot3(vi - xyz(ldg4(f.vel + j)), gr);
            if (dot3(gr, gr) > (R)0) cnt++;
        }
    });
    if (akinci)
        walk<R, 1>(g, bs, pc, xi, c.h, 0, [&](uint32_t j, V3<R> s) {
            const P4<R> pb = ldg4(bpos + j);
            const V3<R> r = s - xyz(pb);
            const R r2 = dot3(r, r);
            if (r2 <= c.cull2) dv += pb.w * dot3(vi, cubic_gradW(c, r, r2));
        });
    return DivSum<R>{dv, cnt};
}

// ---- list walks ------------------------------------------------------------

// DFSPH velocity corrections (MODE 0 warm start, 1 density, 2 divergence),
// as k_dfsph_correct but over the pair lists; kbuf holds this pass's k.
template <typename R, int MODE>
__device__ __forceinline__ V3<R> correct_sum_one(uint32_t i, const Fluid<R>& f, const P4<R>* __restrict__ bpos,
                                                 const GridView& g, const uint32_t* __restrict__ cs,
                                                 const uint32_t* __restrict__ bs, const Consts<R>& c, int akinci,
                                                 const Lists<R>& L)
{
    const uint32_t n = f.n;
    const R* __restrict__ kb_ = L.kbuf;
    const R ki = kb_[i];
    const uint32_t cnt = L.count[i];
    V3<R> sum = {0, 0, 0};
    if (cnt <= L.kmax) {
        const P4<R>* __restrict__ p = L.pairs + i;
#pragma unroll 8
        for (uint32_t k = 0; k < cnt; ++k) {
            const P4<R> q = ldcs4(p + (size_t)k * n);
            const uint32_t j = as_idx(q.w);
            if (!SPH_INDEX_OK(j, n, L.fault)) continue;
            const R kSum = ki + __ldg(kb_ + j);
            if (fabs(kSum) > c.eps) sum = sum + kSum * xyz(q);
        }
        const R kb = MODE == 0 ? c.bwarm * ki : ki;
        if (akinci && fabs(kb) > c.eps) sum = sum + kb * xyz(L.bgrad[i]);
    } else {
        sum = correct_sum_cells<R, MODE>(f, bpos, g, cs, bs, c, akinci, i, ki, kb_);
    }
    return sum;
}

// Velocity update after a correction sum (and the k / kv accumulation).
template <typename R, int MODE>
__device__ __forceinline__ void correct_apply(uint32_t i, const Fluid<R>& f, const Consts<R>& c, R dt, V3<R> sum)
{
    if (MODE == 1) f.kappa[i] += (f.pred[i] - c.density0) * f.alpha[i];
    if (MODE == 2) f.kappav[i] += f.div[i] * f.alpha[i];
    P4<R> v = f.vel[i];
    if (MODE == 0) { v.x -= sum.x * dt; v.y -= sum.y * dt; v.z -= sum.z * dt; }
    else { v.x -= dt * sum.x; v.y -= dt * sum.y; v.z -= dt * sum.z; }
    f.vel[i] = v;
}

// DFSPH velocity corrections (MODE 0 warm start, 1 density, 2 divergence),
// as k_dfsph_correct but over the pair lists; kbuf holds this pass's k.
template <typename R, int MODE>
__global__ void __launch_bounds__(kBlock, 8) k_dfsph_correct_list(Fluid<R> f, const P4<R>* __restrict__ bpos, GridView g,
                                                                  const uint32_t* __restrict__ cs, const uint32_t* __restrict__ bs,
                                                                  Consts<R> c, int akinci, const DevScalars* __restrict__ sc,
                                                                  Lists<R> L)
{
    if (MODE != 0 && !sc->active) return;
    const uint32_t i = gtid();
    if (i >= f.count()) return;
    const V3<R> sum = correct_sum_one<R, MODE>(i, f, bpos, g, cs, bs, c, akinci, L);
    correct_apply<R, MODE>(i, f, c, (R)sc->dt, sum);
}

// Sum over the list of m (v_i - v_j) . gradW_ij plus the boundary term.
template <typename R>
__device__ __forceinline__ R velocity_div_list(const Fluid<R>& f, const Lists<R>& L, uint32_t i, V3<R> vi, int akinci)
{
    const uint32_t n = f.n;
    const uint32_t cnt = L.count[i];
    const P4<R>* __restrict__ p = L.pairs + i;
    R d = 0;
#pragma unroll 8
    for (uint32_t k = 0; k < cnt; ++k) {
        const P4<R> q = ldcs4(p + (size_t)k * n);
        const uint32_t j = as_idx(q.w);
        if (!SPH_INDEX_OK(j, n, L.fault)) continue;
        d += dot3(vi - xyz(ldg4(f.vel + j)), xyz(q));
    }
    if (akinci) d += dot3(vi, xyz(L.bgrad[i]));
    return d;
}

// m (v_i - v_j) . gradW summed over the neighbours (list or fallback walk);
// *nn receives the number of neighbours with a non-zero gradient.
template <typename R>
__device__ __forceinline__ R velocity_div_one(uint32_t i, const Fluid<R>& f, const P4<R>* __restrict__ bpos,
                                              const GridView& g, const uint32_t* __restrict__ cs,
                                              const uint32_t* __restrict__ bs, const Consts<R>& c, int akinci,
                                              const Lists<R>& L, V3<R> vi, uint32_t* nn)
{
    const uint32_t cnt = L.count[i];
    if (cnt <= L.kmax) {
        *nn = cnt;
        return velocity_div_list(f, L, i, vi, akinci);
    }
    const DivSum<R> d = velocity_div_cells(f, bpos, g, cs, bs, c, akinci, i, vi);
    *nn = d.nn;
    return d.dv;
}

// DFSPHSolver::predictDensities over the lists (+ loop control, as
// k_dfsph_predict_density).
template <typename R, bool INITIAL>
__global__ void __launch_bounds__(kBlock, 8) k_dfsph_predict_density_list(Fluid<R> f, const P4<R>* __restrict__ bpos, GridView g,
                                                                       const uint32_t* __restrict__ cs, const uint32_t* __restrict__ bs,
                                                                       Consts<R> c, int akinci, DevScalars* sc, LoopLimits lim,
                                                                       double* partials, cudaGraphConditionalHandle cond,
                                                                       Lists<R> L)
{
    __shared__ double sh[33];
    if (!INITIAL && !sc->active) return;
    const uint32_t i = gtid();
    double err = 0.0;
    if (i < f.count()) {
        const V3<R> vi = xyz(f.vel[i]);
        uint32_t nn;
        const R dc = velocity_div_one(i, f, bpos, g, cs, bs, c, akinci, L, vi, &nn);
        const R dt = (R)sc->dt;
        const R rho = f.rho[i];
        R pred = rho + dc * dt;
        pred = pred < c.density0 ? c.density0 : pred;
        f.pred[i] = pred;
        L.kbuf[i] = (pred - c.density0) * f.alpha[i] / ((dt * dt) * rho);
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

// DFSPHSolver::computeDivergenceError over the lists (+ loop control).
template <typename R, bool INITIAL>
__global__ void __launch_bounds__(kBlock, 8) k_dfsph_divergence_list(Fluid<R> f, const P4<R>* __restrict__ bpos, GridView g,
                                                                  const uint32_t* __restrict__ cs, const uint32_t* __restrict__ bs,
                                                                  Consts<R> c, int akinci, DevScalars* sc, LoopLimits lim,
                                                                  double* partials, cudaGraphConditionalHandle cond,
                                                                  Lists<R> L)
{
    __shared__ double sh[33];
    if (!INITIAL && !sc->active) return;
    const uint32_t i = gtid();
    double err = 0.0;
    if (i < f.count()) {
        const V3<R> vi = xyz(f.vel[i]);
        uint32_t nn;
        R dv = velocity_div_one(i, f, bpos, g, cs, bs, c, akinci, L, vi, &nn);
        const R dt = (R)sc->dt;
        dv = nn < 20u ? (R)0 : (dv < (R)0 ? (R)0 : dv);
        f.div[i] = dv;
        L.kbuf[i] = dv * f.alpha[i] / (dt * f.rho[i]);
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

// The stored lists of the n particles at [base, base + n) of a layout whose
// list slots are `stride` apart (a pooled scene's segment, or a whole scene
// with base 0), keyed by original index: cnt[me] = the particle's neighbour
// count (above kmax when its list overflowed and was not stored) and, with
// off given, the stored neighbours' original indices in list order at
// nbr[off[me]...].
template <typename R>
__global__ void k_pair_lists(uint32_t n, uint32_t base, uint32_t stride, const uint32_t* __restrict__ id, Lists<R> L,
                             const int* __restrict__ off, int* __restrict__ cnt, int* __restrict__ nbr)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const uint32_t i = base + t;
    const uint32_t me = id[i];
    const uint32_t c = L.count[i];
    if (cnt) cnt[me] = (int)c;
    if (off && c <= L.kmax) {
        int* o = nbr + off[me];
        for (uint32_t k = 0; k < c; ++k) o[k] = (int)id[as_idx(L.pairs[(size_t)k * stride + i].w)];
    }
}

// Host side of a pair-list dump (one-scene context and pool alike):
// counts, CSR offsets by original index, and the neighbours.  `launch(off,
// cnt, nbr)` enqueues k_pair_lists on `st`; n = particles.
template <typename Launch>
cudaError_t dump_pair_lists(uint32_t n, uint32_t kmax, cudaStream_t st, Launch&& launch, int* count, int* off, int* nbr,
                            long long* total)
{
    int* dc = nullptr;
    int* doff = nullptr;
    int* dn = nullptr;
    std::vector<int> hc(n), ho(n + 1);
    long long a = 0;
    cudaError_t e = cudaMalloc((void**)&dc, sizeof(int) * (n ? n : 1));
    if (e == cudaSuccess && n) {
        launch((const int*)nullptr, dc, (int*)nullptr);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && n) e = cudaMemcpyAsync(hc.data(), dc, sizeof(int) * n, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) {
        for (uint32_t i = 0; i < n; ++i) {
            ho[i] = (int)a;
            a += (uint32_t)hc[i] <= kmax ? hc[i] : 0;
        }
        ho[n] = (int)a;
        if (total) *total = a;
        if (count && n) std::memcpy(count, hc.data(), sizeof(int) * n);
        if (off) std::memcpy(off, ho.data(), sizeof(int) * (n + 1));
    }
    if (e == cudaSuccess && nbr && a) {
        e = cudaMalloc((void**)&doff, sizeof(int) * (n + 1));
        if (e == cudaSuccess) e = cudaMalloc((void**)&dn, sizeof(int) * (size_t)a);
        if (e == cudaSuccess) e = cudaMemcpyAsync(doff, ho.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) {
            launch((const int*)doff, (int*)nullptr, dn);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaMemcpyAsync(nbr, dn, sizeof(int) * (size_t)a, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    }
    cudaStreamSynchronize(st);
    cudaFree(dc);
    cudaFree(doff);
    cudaFree(dn);
    return e;
}

// Warm-start scaling (as k_dfsph_predict_v_warm) writing k to the list
// pass's kbuf.
template <typename R>
__global__ void k_dfsph_predict_v_warm_list(Fluid<R> f, Consts<R> c, const DevScalars* __restrict__ sc, R* __restrict__ kbuf)
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
    kbuf[i] = -mx / ts2;
    f.kappa[i] = 0;
}

}  // namespace sph
