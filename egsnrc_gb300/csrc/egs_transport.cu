// GB300 transport kernels and the C-ABI engine behind include/egsgpu.h.
//
// Histories run as a wavefront over per-type SoA particle queues in HBM:
//   k_source    one thread per history: samples the source particle and
//               places it on the phantom surface (egs++ simulateSingleShower,
//               egs_application.cpp:919-959, egs_nd_geometry.h:1281-1379)
//   k_photon    persistent warps; each iteration moves one photon through one
//               voxel (or to its interaction) and samples the interaction
//               (PHOTON, src/egsnrc.mortran:6439-6641); electrons are pushed
//               to the electron queue
//   k_electron  persistent warps; each iteration takes one condensed-history
//               step (ELECTR, src/egsnrc.mortran:985-1821) and, when the
//               sub-threshold energy-loss budget is used up, the discrete
//               interaction; photons go to the next photon queue, delta rays
//               to the next electron queue
//   k_batch     folds the batch tally into the per-voxel sum and sum of squares
// Energy deposits are accumulated per thread while a particle stays in one
// voxel and flushed with one FP64 atomic (tallies are L2-resident).
// The file builds the FP32 engine and the C ABI; egs_transport_f64.cu builds
// the FP64 engine from it (see EGSGPU_TU below).
// Paths in comments are relative to the EGSnrc HEN_HOUSE directory.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <new>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/egsgpu.h"
// This file is compiled twice: as itself (the FP32 engine and the C ABI) and,
// through egs_transport_f64.cu, as the FP64 engine without fused multiply-adds.
// Each compilation keeps its kernels, device constants and engine in its own
// namespace, EGSGPU_TU, so that the two share no symbol.
#ifndef EGSGPU_TU
#define EGSGPU_TU tu32
#endif
#include "egs_device.cuh"
#include "egs_hatch.h"
#include "egs_physics.cuh"

namespace cg = cooperative_groups;

namespace egsgpu {

static __host__ __device__ __noinline__ uint4 philox_block(uint32_t b, uint32_t s0, uint32_t s1, uint32_t k0,
                                                           uint32_t k1) {
    uint32_t o[4];
    philox10(b, s0, s1, 0u, k0, k1, o);
    return make_uint4(o[0], o[1], o[2], o[3]);
}

namespace EGSGPU_TU {

__constant__ MedScalars<float> c_med_f[MAXMED];
__constant__ MedScalars<double> c_med_d[MAXMED];
template <class Real> __device__ inline const MedScalars<Real> &cmed(int m);
template <> __device__ inline const MedScalars<float> &cmed<float>(int m) { return c_med_f[m]; }
template <> __device__ inline const MedScalars<double> &cmed<double>(int m) { return c_med_d[m]; }

// Counters: 0 photon steps, 1 electron steps, 2 pushes, 3 interactions.
// A particle that needs more than STEP_CAP steps is retired and reported
// (EGSGPU_ERR_LOOP); no physical history comes near the default.

enum { CNT_PSTEP = 0, CNT_ESTEP = 1, CNT_PUSH = 2, CNT_INTER = 3, CNT_EPUSH = 4, CNT_EINTER = 5,
       CNT_PLANES = 6, CNT_PITER = 7, CNT_ELANES = 8, CNT_EITER = 9, CNT_EWIDE = 10, CNT_N = 12 };

template <class Real>
struct Params {
    Tables<Real> T;
    Geom<Real> G;
    Queue<Real> pin, ein, pout, eout;    // consumed / produced queues
    double *dose;                         // batch tally per voxel
    // several phantoms in one run (Multi kernels): per-phantom geometry,
    // Philox seed and source, the phantoms' first global voxel indices
    // (nprob + 1 entries, ascending) and, for the current batch, the prefix
    // sums of the phantoms' history counts and their first history indices
    const Geom<Real> *probs;
    const uint32_t *pseeds;
    const Source *psrc;
    const int *pvoff;
    const long long *pprefix, *pfirst;
    int nprob;
    // seed-replay adjoint: dL/dE per voxel (also weights the per-history
    // tally when set), per-history weighted deposits G_h of the replayed
    // histories (index hist - hist_first) and the dL/d(rhor) accumulator
    const double *wvox;
    const double *hist_G;
    double *grad;
    double *hist_tally;                   // optional per-history deposits
    long long hist_first, hist_n;
    double *energy;                       // [0] deposited, [1] escaped
    unsigned long long *counters;         // CNT_*
    int *error;                           // [0] capacity, [1] loop cap
    unsigned *peak;                       // largest queue length seen (autotuner input)
    uint32_t seed;
    int requeue_lanes;                    // park survivors of warps this sparse (0 = never)
    int inter_batch;                      // electron lanes due to interact before the warp samples them
    int inter_batch_p;                    // the same for photon lanes
};

// A warp whose queue is exhausted parks its particles in the next queue once
// this few of its lanes are still busy (only when the launch is large enough
// for the next round to refill warps).
constexpr unsigned REQUEUE_MIN = 32768;
constexpr int LSTACK = 6;   // per-thread LIFO depth for charged secondaries
// A photon lane crosses up to this many voxels per iteration of the persistent
// loop before the warp's bookkeeping (refill, interaction batching) runs again.
constexpr int PHOTON_HOPS = 16;
constexpr int INTER_MAXWAIT = 24;   // longest wait of a lane due to interact
// Random numbers made present ahead of an electron step or an interaction
// batch: a PRESTA-II step with the q-surface sampler takes 11 (two
// deflections, two azimuths, the lateral displacement), plus one for a new
// step length and one for the fictitious-cross-section test.
constexpr unsigned RNG_AHEAD = 13;
constexpr int MAX_BLOCK = 128;      // launch bound of the transport kernels (threads per CTA)
constexpr double VERY_FAR = 1e30;   // egs++ veryFar (egs++/egs_functions.h:105)
// Distance to a voxel face (cm) within which an FP32 electron step is computed
// in FP64 when the precision split is on: 2^-12 cm, about 250 FP32 units in
// the last place of a coordinate of 16 cm.
constexpr double NEAR_FACE = 1.0 / 4096.0;

// ------------------------------------------------------------- tallies ----
template <class Real>
struct Acc {
    int ir;
    uint32_t hist;
    Real e;   // deposits of one particle's visit to one voxel
};

template <class Real>
__device__ inline void acc_flush(const Params<Real> &P, Acc<Real> &a) {
    if (a.ir >= 0 && a.e > 0) {
        atomicAdd(P.dose + a.ir, (double)a.e);
        if (P.hist_tally) {
            long long i = (long long)a.hist - P.hist_first;
            if (i >= 0 && i < P.hist_n) atomicAdd(P.hist_tally + i, P.wvox ? P.wvox[a.ir] * (double)a.e : (double)a.e);
        }
    }
    a.e = 0;
    a.ir = -1;
}
template <class Real>
__device__ inline void deposit(const Params<Real> &P, Acc<Real> &a, int ir, uint32_t hist, Real e) {
    if (ir < 0 || !(e > 0)) return;
    if (ir != a.ir || hist != a.hist) {
        acc_flush(P, a);
        a.ir = ir;
        a.hist = hist;
    }
    a.e += e;
}

// Gradient contributions of one particle's visit to one voxel, flushed with
// one FP64 atomic when the voxel changes (adjoint replay only).
template <class Real>
struct AccG {
    int ir;
    Real g;
};
template <class Real>
__device__ inline void gflush(const Params<Real> &P, AccG<Real> &a) {
    if (a.ir >= 0 && a.g != 0) atomicAdd(P.grad + a.ir, (double)a.g);
    a.g = 0;
    a.ir = -1;
}
template <class Real>
__device__ inline void gadd(const Params<Real> &P, AccG<Real> &a, int ir, Real g) {
    if (ir != a.ir) {
        gflush(P, a);
        a.ir = ir;
    }
    a.g += g;
}
// Pathwise derivative of an electron track's continuous energy loss (the
// adjoint's electron term).  With a condensed-history step's random numbers
// fixed in mass units, raising rhor_j shortens the track's path inside voxel
// j, so every later voxel-face crossing moves along the track by
// c_j[a] / (rhor_j u[a]) -- c_j the track's chord vector inside j so far, a
// the axis of the crossed face, u the direction at the crossing -- and the
// energy lost over that shift (dE/dx in the voxel being left) moves from the
// voxel entered (weight w_b; 0 outside the phantom) to the one left (w_a).
// Each visit to a voxel keeps its chord vector and accumulates
// K = sum over later crossings of (w_a - w_b) dE/dx c[a] / u[a]; the track's
// end adds K / rhor to dL/d(rhor) of the visited voxel.  ELIST visits are
// kept per electron; a longer track flushes its oldest part early (without
// the crossings that follow).  Displacements of discrete-interaction points
// and of the end-of-track deposit are not followed.
constexpr int ELIST = 48;
template <class Real>
struct EList {
    int n;
    int v[ELIST];
    Real c[ELIST][3];
    Real k[ELIST];
};
template <class Real>
__device__ inline void elist_flush(const Params<Real> &P, EList<Real> &L) {
    for (int i = 0; i < L.n; ++i)
        if (L.k[i] != 0) atomicAdd(P.grad + L.v[i], (double)(L.k[i] / P.G.rhor[L.v[i]]));
    L.n = 0;
}
// a step of displacement d inside voxel ir
template <class Real>
__device__ inline void elist_step(const Params<Real> &P, EList<Real> &L, int ir, Real dx, Real dy, Real dz) {
    if (L.n == 0 || L.v[L.n - 1] != ir) {
        if (L.n == ELIST) elist_flush(P, L);
        L.v[L.n] = ir;
        L.c[L.n][0] = 0; L.c[L.n][1] = 0; L.c[L.n][2] = 0;
        L.k[L.n] = 0;
        ++L.n;
    }
    L.c[L.n - 1][0] += dx; L.c[L.n - 1][1] += dy; L.c[L.n - 1][2] += dz;
}
// a crossing of a face normal to `axis` with direction component ua
template <class Real>
__device__ inline void elist_cross(EList<Real> &L, int axis, Real ua, Real coef) {
    if (ua == 0) return;
    const Real f = coef / ua;
    for (int i = 0; i < L.n; ++i) L.k[i] += f * L.c[i][axis];
}
// G_h of the particle's history in an adjoint replay
template <class Real>
__device__ inline Real hist_weight(const Params<Real> &P, const Particle<Real> &p) {
    long long i = (long long)p.rng.hist - P.hist_first;
    return (i >= 0 && i < P.hist_n) ? (Real)P.hist_G[i] : (Real)0;
}

// ------------------------------------------------------------- queues ----
template <class Real>
__device__ inline void q_store(const Queue<Real> &q, unsigned i, const Particle<Real> &p) {
    q.x[i] = p.x; q.y[i] = p.y; q.z[i] = p.z;
    q.u[i] = p.u; q.v[i] = p.v; q.w[i] = p.w;
    q.E[i] = p.E; q.wt[i] = p.wt; q.ir[i] = p.ir;
    if (q.iq) q.iq[i] = (int8_t)p.iq;
    q.hist[i] = p.rng.hist; q.n[i] = p.rng.n; q.sid[i] = p.rng.sid;
    q.st[i] = 0;
}
template <class Real>
__device__ inline void q_load(const Queue<Real> &q, unsigned i, uint32_t seed, Particle<Real> &p) {
    p.x = q.x[i]; p.y = q.y[i]; p.z = q.z[i];
    p.u = q.u[i]; p.v = q.v[i]; p.w = q.w[i];
    p.E = q.E[i]; p.wt = q.wt[i]; p.ir = q.ir[i];
    p.iq = q.iq ? (int)q.iq[i] : 0;
    p.rng.init(seed, q.hist[i], q.sid[i], q.n[i]);
}
// The phantom holding global voxel `ir` (largest k with pvoff[k] <= ir).
template <class Real>
__device__ inline int phantom_of(const Params<Real> &P, int ir) {
    int lo = 0, hi = P.nprob;
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (ir >= P.pvoff[mid]) lo = mid; else hi = mid;
    }
    return lo;
}
// Loads queue record i; in a multi-phantom run the particle's phantom (and
// with it its Philox seed) follows from its voxel index.
template <class Real, bool Multi>
__device__ inline void load_particle(const Params<Real> &P, const Queue<Real> &q, unsigned i, Particle<Real> &p) {
    if (Multi) {
        int k = phantom_of(P, q.ir[i]);
        q_load(q, i, P.pseeds[k], p);
        p.pb = k;
    } else {
        q_load(q, i, P.seed, p);
        p.pb = 0;
    }
}
template <class Real, bool Multi>
__device__ inline const Geom<Real> &geom_of(const Params<Real> &P, int pb) {
    return Multi ? P.probs[pb] : P.G;
}
// Warp-aggregated append: the lanes that reach the push together share one
// atomic on the queue counter.  Returns the slot, or ~0u when the queue is full.
template <class Real>
__device__ inline unsigned q_slot(const Params<Real> &P, const Queue<Real> &q) {
    cg::coalesced_group g = cg::coalesced_threads();
    unsigned base = 0;
    if (g.thread_rank() == 0) base = atomicAdd(q.count, (unsigned)g.size());
    base = g.shfl(base, 0);
    unsigned i = base + g.thread_rank();
    if (i < q.capacity) return i;
    atomicExch(P.error + 0, 1);
    return ~0u;
}
template <class Real>
__device__ inline void q_push(const Params<Real> &P, const Queue<Real> &q, const Particle<Real> &p,
                              unsigned long long &npush) {
    unsigned i = q_slot(P, q);
    if (i != ~0u) {
        q_store(q, i, p);
        ++npush;
    }
}

// ANNIH_AT_REST (src/egsnrc.mortran:186-223): two back-to-back photons of
// rest energy, the first continuing the positron's stream.
template <class Real>
__device__ inline void annih_at_rest(const Params<Real> &P, const Queue<Real> &qp, Particle<Real> &p,
                                     unsigned long long &npush, int &err) {
    const Real rm = (Real)RM;
    Real costhe = urand<Real>(p.rng);
    costhe = 2 * costhe - 1;
    Real sinthe = dsqrt(dmax((Real)0, (1 - costhe) * (1 + costhe)));
    Azim<Real> az = azimuth<Real>(p.rng, err);
    Particle<Real> g1 = p, g2 = p;
    g1.E = rm; g1.iq = 0; g1.u = sinthe * az.c; g1.v = sinthe * az.s; g1.w = costhe;
    g2.rng.init(p.rng.seed, p.rng.hist, child_sid(p.rng.sid, p.rng.n, 0), 0u);
    g2.E = rm; g2.iq = 0; g2.u = -g1.u; g2.v = -g1.v; g2.w = -g1.w;
    q_push(P, qp, g1, npush);
    q_push(P, qp, g2, npush);
}

// Queue a new electron/positron, or -- when it is already at or below the
// cut-off -- do its :ECUT-DISCARD: right here (deposit, and annihilation at
// rest for a positron, on its own stream): what ELECTR would do first.
template <class Real>
__device__ inline void push_charged(const Params<Real> &P, const Queue<Real> &qe, const Queue<Real> &qp,
                                    Particle<Real> &q, Acc<Real> &acc, unsigned long long &npush,
                                    double &edep_tot, int &err) {
    if (q.E <= P.T.ecut) {
        Real edep = q.E - (Real)RM;
        deposit(P, acc, q.ir, q.rng.hist, edep * q.wt);
        edep_tot += (double)(edep * q.wt);
        if (q.iq > 0) annih_at_rest(P, qp, q, npush, err);
        return;
    }
    q_push(P, qe, q, npush);
}

// ----------------------------------------------------------- geometry ----
// EGS_XYZGeometry::howfar (egs++/geometry/egs_nd_geometry/egs_nd_geometry.h:963-1104)
template <class Real>
__device__ inline int howfar(const Geom<Real> &G, int ireg, Real x, Real y, Real z, Real u, Real v, Real w,
                             Real &t, int &axis) {
    const int loc = ireg - G.voff;
    int iz = fdiv(loc, G.mnxy, G.lnxy), ir = loc - iz * G.nxy, iy = fdiv(ir, G.mnx, G.lnx), ix = ir - iy * G.nx;
    int inew = ireg;
    if (u > 0) {
        Real d = (G.xb[ix + 1] - x) / u;
        if (d <= t) { t = (d <= G.bt) ? G.hbt : d; inew = (ix + 1 < G.nx) ? ireg + 1 : -1; axis = 0; }
    } else if (u < 0) {
        Real d = (G.xb[ix] - x) / u;
        if (d <= t) { t = (d <= G.bt) ? G.hbt : d; inew = (ix - 1 >= 0) ? ireg - 1 : -1; axis = 0; }
    }
    if (v > 0) {
        Real d = (G.yb[iy + 1] - y) / v;
        if (d <= t) { t = (d <= G.bt) ? G.hbt : d; inew = (iy + 1 < G.ny) ? ireg + G.nx : -1; axis = 1; }
    } else if (v < 0) {
        Real d = (G.yb[iy] - y) / v;
        if (d <= t) { t = (d <= G.bt) ? G.hbt : d; inew = (iy - 1 >= 0) ? ireg - G.nx : -1; axis = 1; }
    }
    if (w > 0) {
        Real d = (G.zb[iz + 1] - z) / w;
        if (d <= t) { t = (d <= G.bt) ? G.hbt : d; inew = (iz + 1 < G.nz) ? ireg + G.nxy : -1; axis = 2; }
    } else if (w < 0) {
        Real d = (G.zb[iz] - z) / w;
        if (d <= t) { t = (d <= G.bt) ? G.hbt : d; inew = (iz - 1 >= 0) ? ireg - G.nxy : -1; axis = 2; }
    }
    return inew;
}
template <class Real>
__device__ inline int howfar(const Geom<Real> &G, int ireg, Real x, Real y, Real z, Real u, Real v, Real w,
                             Real &t) {
    int axis;
    return howfar(G, ireg, x, y, z, u, v, w, t, axis);
}
// EGS_XYZGeometry::hownear (egs_nd_geometry.h:1106-1122)
template <class Real>
__device__ inline Real hownear(const Geom<Real> &G, int ireg, Real x, Real y, Real z) {
    const int loc = ireg - G.voff;
    int iz = fdiv(loc, G.mnxy, G.lnxy), ir = loc - iz * G.nxy, iy = fdiv(ir, G.mnx, G.lnx), ix = ir - iy * G.nx;
    Real t = dmin(x - G.xb[ix], G.xb[ix + 1] - x);
    t = dmin(t, dmin(y - G.yb[iy], G.yb[iy + 1] - y));
    t = dmin(t, dmin(z - G.zb[iz], G.zb[iz + 1] - z));
    return t;
}
// EGS_PlanesT::isWhere with EGS_BaseGeometry::findRegion (egs++/geometry/
// egs_planes/egs_planes.h:301-311, egs++/egs_base_geometry.h:178-190): the
// slab of b[0..n] holding x, -1 outside; a point on an interior plane belongs
// to the slab below it.
template <class Real>
__device__ inline int plane_where(const Real *b, int n, Real x) {
    if (x < b[0] || x > b[n]) return -1;
    int lo = 0, hi = n;
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (x <= b[mid]) hi = mid; else lo = mid;
    }
    return hi - 1;
}
// EGS_XYZGeometry::howfarFromOut (egs_nd_geometry.h:1281-1379): the region a
// particle outside the phantom at `pos` enters along `dir` within t (the
// x faces are tried first, then y, then z), or -1; t receives the distance.
// Positions are FP64 in both builds, as in the source kernel.
template <class Real>
__device__ inline int howfar_from_out(const Geom<Real> &G, const double pos[3], const double dir[3], double &t) {
    const Real *pl[3] = {G.xb, G.yb, G.zb};
    const int nn[3] = {G.nx, G.ny, G.nz};
    for (int a = 0; a < 3; ++a) {
        int i = -1;
        double t1 = 0;
        const double b0 = (double)pl[a][0], bn = (double)pl[a][nn[a]];
        if (pos[a] <= b0 && dir[a] > 0) { t1 = (b0 - pos[a]) / dir[a]; i = 0; }
        else if (pos[a] >= bn && dir[a] < 0) { t1 = (bn - pos[a]) / dir[a]; i = nn[a] - 1; }
        if (i < 0 || !(t1 <= t)) continue;
        const double q[3] = {pos[0] + dir[0] * t1, pos[1] + dir[1] * t1, pos[2] + dir[2] * t1};
        int idx[3];
        bool ok = true;
        for (int c = 0; c < 3 && ok; ++c) {
            if (c == a) idx[c] = i;
            else { idx[c] = plane_where(pl[c], nn[c], (Real)q[c]); ok = idx[c] >= 0; }
        }
        if (!ok) continue;
        const int inew = G.voff + idx[0] + idx[1] * G.nx + idx[2] * G.nxy;
        if (t1 < (double)G.bt) {   // entering at an edge: the step may end at once
            Real tt = (Real)t1;
            int itest = howfar(G, inew, (Real)q[0], (Real)q[1], (Real)q[2], (Real)dir[0], (Real)dir[1], (Real)dir[2], tt);
            if (itest == -1 && tt < G.bt) return -1;
            t1 = (double)tt;
        }
        t = t1;
        return inew;
    }
    return -1;
}


// ------------------------------------------------ HOWFARLESS geometry ----
// DOSXYZnrc ihowfarless = 1 in a homogeneous phantom (dosxyznrc.mortran
// HOWFAR :4177-4200, HOWNEAR :4351-4355): particles see only the phantom's
// outer faces; voxels matter for scoring alone.
template <class Real>
__device__ inline Real hfl_dist_out(const Geom<Real> &G, const Particle<Real> &p) {
    Real d = (Real)1e20;
    if (p.u > 0) d = dmin(d, (G.xb[G.nx] - p.x) / p.u); else if (p.u < 0) d = dmin(d, (G.xb[0] - p.x) / p.u);
    if (p.v > 0) d = dmin(d, (G.yb[G.ny] - p.y) / p.v); else if (p.v < 0) d = dmin(d, (G.yb[0] - p.y) / p.v);
    if (p.w > 0) d = dmin(d, (G.zb[G.nz] - p.z) / p.w); else if (p.w < 0) d = dmin(d, (G.zb[0] - p.z) / p.w);
    return d;
}
template <class Real>
__device__ inline Real hfl_hownear(const Geom<Real> &G, const Particle<Real> &p) {
    Real t = dmin(p.x - G.xb[0], G.xb[G.nx] - p.x);
    t = dmin(t, dmin(p.y - G.yb[0], G.yb[G.ny] - p.y));
    return dmin(t, dmin(p.z - G.zb[0], G.zb[G.nz] - p.z));
}
template <class Real>
__device__ inline int hfl_howfar(const Geom<Real> &G, const Particle<Real> &p, Real &t) {
    Real d = hfl_dist_out(G, p);
    if (d <= t) { t = (d <= G.bt) ? G.hbt : d; return -1; }
    return p.ir;
}
template <class Real>
__device__ inline int hfl_index(const Real *b, int n, Real v) {
    if (v <= b[0]) return 0;
    if (v >= b[n]) return n - 1;
    int lo = 0, hi = n;
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (v < b[mid]) hi = mid; else lo = mid;
    }
    return lo;
}
template <class Real>
__device__ inline int hfl_locate(const Geom<Real> &G, Real x, Real y, Real z) {
    return hfl_index(G.xb, G.nx, x) + hfl_index(G.yb, G.ny, y) * G.nx + hfl_index(G.zb, G.nz, z) * G.nxy;
}
// HOWFARLESS dose deposition of one charged-particle step
// (dosxyznrc.mortran:3569-3760): the step from xi0 / ui0 to the particle's
// end point and direction, of path length tv, becomes two straight segments
// joined at a hinge placed from the initial or (with equal probability) the
// final direction -- one straight segment for a step without multiple
// scattering -- and its energy edep is shared among the voxels the segments
// cross in proportion to the path length in each.  p.ir holds the start.
// Returns the voxel at the end of the segments, or -1 when they leave the
// phantom; `lost` is then the energy past that point, not deposited.
template <class Real>
__device__ int hfl_hinge(const Params<Real> &P, Acc<Real> &acc, const Geom<Real> &G, Particle<Real> &p,
                         const Real xi0[3], const Real ui0[3], Real tv, bool ch_step, Real edep, Real &lost, int &err) {
    lost = 0;
    const int loc = p.ir;
    int iz = fdiv(loc, G.mnxy, G.lnxy), rr = loc - iz * G.nxy, iy = fdiv(rr, G.mnx, G.lnx), ix = rr - iy * G.nx;
    if (p.x > G.xb[ix] && p.x < G.xb[ix + 1] && p.y > G.yb[iy] && p.y < G.yb[iy + 1] && p.z > G.zb[iz] &&
        p.z < G.zb[iz + 1]) {
        deposit(P, acc, loc, p.rng.hist, edep * p.wt);
        return loc;
    }
    const Real d[3] = {p.x - xi0[0], p.y - xi0[1], p.z - xi0[2]};
    const Real d2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    Real t0 = tv, t1 = 0;
    Real u0[3] = {ui0[0], ui0[1], ui0[2]}, u1[3] = {0, 0, 0};
    if (ch_step) {
        if (urand<Real>(p.rng) < (Real)0.5) {   // hinge from the initial direction
            Real c = 1 - (d[0] * u0[0] + d[1] * u0[1] + d[2] * u0[2]) / tv;
            if (c < (Real)1e-3) {
                t0 = dsqrt(d2);
                for (int k = 0; k < 3; ++k) u0[k] = d[k] / t0;
            } else {
                t0 = (tv * tv - d2) / (2 * tv * c);
                t1 = tv - t0;
                for (int k = 0; k < 3; ++k) u1[k] = (d[k] - t0 * u0[k]) / (tv - t0);
            }
        } else {                                 // hinge from the final direction
            u1[0] = p.u; u1[1] = p.v; u1[2] = p.w;
            Real c = 1 - (d[0] * u1[0] + d[1] * u1[1] + d[2] * u1[2]) / tv;
            if (c < (Real)1e-3) {
                t0 = dsqrt(d2);
                for (int k = 0; k < 3; ++k) u0[k] = d[k] / t0;
            } else {
                t1 = (tv * tv - d2) / (2 * tv * c);
                t0 = tv - t1;
                for (int k = 0; k < 3; ++k) u0[k] = (d[k] - t1 * u1[k]) / (tv - t1);
            }
        }
    }
    const Real frac = edep / (t0 + t1);
    const Real *B[3] = {G.xb, G.yb, G.zb};
    const int n[3] = {G.nx, G.ny, G.nz}, stride[3] = {1, G.nx, G.nxy};
    int idx[3] = {ix, iy, iz}, cur = loc;
    Real pos[3] = {xi0[0], xi0[1], xi0[2]}, done = 0;
    const int cap = G.nx + G.ny + G.nz + 8;
#pragma unroll 1
    for (int s = 0; s < 2; ++s) {
        const Real ts = s ? t1 : t0;
        if (!(ts > 0)) continue;
        const Real *u = s ? u1 : u0;
        if (s == 1)
            for (int k = 0; k < 3; ++k) pos[k] += u0[k] * t0;
        int dir[3];
        Real dist[3], inv[3];
        for (int k = 0; k < 3; ++k) {
            if (u[k] > 0) { inv[k] = 1 / dabs(u[k]); dir[k] = 1; dist[k] = (B[k][idx[k] + 1] - pos[k]) * inv[k]; }
            else if (u[k] < 0) { inv[k] = 1 / dabs(u[k]); dir[k] = -1; dist[k] = (pos[k] - B[k][idx[k]]) * inv[k]; }
            else { inv[k] = 0; dir[k] = 0; dist[k] = (Real)1e20; }
        }
        Real walked = 0;
        for (int it = 0;; ++it) {
            if (it > cap) { err = 1; break; }
            Real dmax = ts - walked, dl;
            int a = -1;
            if (dist[0] < dist[1] && dist[0] < dist[2] && dist[0] < dmax) a = 0;
            else if (dist[1] < dist[2] && dist[1] < dmax) a = 1;
            else if (dist[2] < dmax) a = 2;
            bool out = false;
            int next = cur;
            if (a < 0) dl = dmax;
            else {
                dl = dist[a];
                idx[a] += dir[a];
                if (idx[a] >= 0 && idx[a] < n[a]) {
                    for (int k = 0; k < 3; ++k) if (k != a) dist[k] -= dl;
                    next = cur + dir[a] * stride[a];
                    dist[a] = (B[a][idx[a] + 1] - B[a][idx[a]]) * inv[a];
                } else out = true;
            }
            deposit(P, acc, cur, p.rng.hist, dl * frac * p.wt);
            done += dl;
            walked += dl;
            if (out) { lost = edep - done * frac; return -1; }
            cur = next;
            if (walked >= ts) break;
        }
    }
    return cur;
}

// ------------------------------------------------------------- source ----
// One thread per history.  A single-phantom run transports histories
// first + t; a multi-phantom run maps t to phantom k and history
// pfirst[k] + (first + t - pprefix[k]) of that phantom, so every phantom sees
// the histories (and random numbers) of a run of its own.
template <class Real, bool Multi>
__global__ void k_source(Params<Real> P, Source S0, long long first, long long n) {
    long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= n) return;
    int k = 0;
    uint32_t hist = (uint32_t)(first + t), seed = P.seed;
    if (Multi) {
        long long g = first + t;
        int lo = 0, hi = P.nprob;
        while (hi - lo > 1) {
            int mid = (lo + hi) >> 1;
            if (g >= P.pprefix[mid]) lo = mid; else hi = mid;
        }
        k = lo;
        hist = (uint32_t)(P.pfirst[k] + (g - P.pprefix[k]));
        seed = P.pseeds[k];
    }
    const Source &S = Multi ? P.psrc[k] : S0;
    Particle<Real> p;
    p.rng.init(seed, hist, 0ull, 0u);
    p.pb = k;
    p.wt = 1;
    double x = S.pos[0], y = S.pos[1], z = S.pos[2];
    double u = S.dir[0], v = S.dir[1], w = S.dir[2];
    int charge = S.charge;
    if (S.shape == 1) {
        x = S.xmin + (S.xmax - S.xmin) * (double)urand<Real>(p.rng);
        y = S.ymin + (S.ymax - S.ymin) * (double)urand<Real>(p.rng);
    }
    double ek;
    if (S.shape == 2) {   // phase-space particle (egs_phsp_source.cpp:296-320)
        const float *q = S.phsp + 7 * (((long long)hist / (S.recycle + 1)) % S.nphsp);
        charge = (int)q[0];
        ek = q[1];
        x += q[2]; y += q[3];
        u = q[4]; v = q[5];
        double a = u * u + v * v;
        w = a < 1 ? sqrt(1 - a) : 0.0;
        if (q[6] < 0) w = -w;
        p.wt = (Real)(fabs((double)q[6]) / (S.recycle + 1));
        if (S.has_rot) {   // EGS_TransformedSource: x' = R (x, y, 0) + t, u' = R u
            const double *R = S.rot, px = q[2], py = q[3], u0 = u, v0 = v, w0 = w;
            x = S.pos[0] + (R[0] * px + R[1] * py);
            y = S.pos[1] + (R[3] * px + R[4] * py);
            z = S.pos[2] + (R[6] * px + R[7] * py);
            u = R[0] * u0 + R[1] * v0 + R[2] * w0;
            v = R[3] * u0 + R[4] * v0 + R[5] * w0;
            w = R[6] * u0 + R[7] * v0 + R[8] * w0;
        }
    } else if (S.spectrum == 0) ek = S.energy;
    else {
        double aj = (double)urand<Real>(p.rng) * S.nbins;
        int j = (int)aj;
        aj -= j;
        if (aj > S.wi[j]) j = S.bin[j];
        ek = S.edges[j] + (S.edges[j + 1] - S.edges[j]) * (double)urand<Real>(p.rng);
    }
    p.iq = charge;
    p.E = (Real)(p.iq == 0 ? ek : ek + RM);
    const Geom<Real> &G = geom_of<Real, Multi>(P, k);
    // EGS_Application::simulateSingleShower (egs_application.cpp:938-945):
    // isWhere, then howfarFromOut with t = veryFar and x += u t, in FP64
    int ix = plane_where(G.xb, G.nx, (Real)x), iy = plane_where(G.yb, G.ny, (Real)y), iz = plane_where(G.zb, G.nz, (Real)z);
    int ir = (ix >= 0 && iy >= 0 && iz >= 0) ? G.voff + ix + iy * G.nx + iz * G.nxy : -1;
    if (ir < 0) {
        const double pos[3] = {x, y, z}, dir[3] = {u, v, w};
        double t = VERY_FAR;
        ir = howfar_from_out(G, pos, dir, t);
        if (ir >= 0) { x += u * t; y += v * t; z += w * t; }
    }
    if (ir < 0) return;
    p.x = (Real)x; p.y = (Real)y; p.z = (Real)z;
    p.u = (Real)u; p.v = (Real)v; p.w = (Real)w;
    p.ir = ir;
    unsigned long long np = 0;
    if (p.iq == 0) q_push(P, P.pout, p, np);
    else q_push(P, P.eout, p, np);
}

// ------------------------------------------------------------- photon ----
template <class Real>
struct PhotonState {
    int state;            // 0 new energy, 1 new medium, 2 transport
    int medium, nsteps;
    Real rhor, gle, dpmfp, gmfpr0, cohfac;
    int lgle;
};

// Adj: adjoint replay.  Each photon path segment of dpmfp mean free paths in
// voxel v adds -G_h * dpmfp / rhor_v to dL/d(rhor_v) and each interaction in
// v adds G_h / rhor_v: the score of the path's likelihood (all attenuation
// coefficients scale with rhor, PHOTON's GMFP = GMFPR0 / RHOF), times the
// history's weighted deposit G_h.
// HFL: HOWFARLESS transport (one flight to the interaction or out of the
// phantom; the voxel is located where the photon interacts).
// FP32: eight CTAs per SM (at most 64 registers).  The photon loop is latency
// bound and gains more from resident warps than it loses to its few spills
// (+5% on slab phantoms over the unbounded 94-register build); the FP64 build
// would spill ~1 KB per thread at that bound and keeps its registers.
template <class Real, bool Multi, bool Adj = false, bool HFL = false>
__global__ void __launch_bounds__(MAX_BLOCK, sizeof(Real) == 4 ? 8 : 1) k_photon(Params<Real> P) {
    const Tables<Real> &T = P.T;
    const Geom<Real> &G = P.G;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned nq = *P.pin.count < P.pin.capacity ? *P.pin.count : P.pin.capacity;
    if (threadIdx.x == 0 && blockIdx.x == 0) atomicMax(P.peak, *P.pin.count);
    __shared__ unsigned s_dummy;
    (void)s_dummy;
    Particle<Real> p;
    PhotonState<Real> s;
    Acc<Real> acc{-1, 0u, (Real)0};
    AccG<Real> ga{-1, (Real)0};
    Real Gh = 0;
    bool alive = false, exhausted = false;
    unsigned long long nstep = 0, npush = 0, ninter = 0, lanes = 0, iters = 0;
    int inter_wait = 0;   // warp-uniform iterations since the first lane became due
    double edep_tot = 0, esc_tot = 0;
    int err = 0;
    const Real rm = (Real)RM;
    const bool requeue = P.requeue_lanes > 0 && nq >= REQUEUE_MIN;
    while (true) {
        if (exhausted && requeue) {
            unsigned busy = __ballot_sync(0xffffffffu, alive);
            if (__popc(busy) <= P.requeue_lanes) {   // park the survivors and retire the warp
                if (alive) {
                    unsigned i = q_slot(P, P.pout);
                    if (i != ~0u) {
                        q_store(P.pout, i, p);
                        if (s.state == 3) P.pout.st[i] = 3;
                        else if (s.state != 0) { P.pout.st[i] = 1; P.pout.aux0[i] = s.dpmfp; }
                    }
                }
                break;
            }
        }
        unsigned need = __ballot_sync(0xffffffffu, !alive);
        if (need && !exhausted) {
            unsigned base = 0;
            if (lane == (unsigned)(__ffs(need) - 1)) base = atomicAdd(P.pin.count + 1, (unsigned)__popc(need));
            base = __shfl_sync(0xffffffffu, base, __ffs(need) - 1);
            if (base >= nq) exhausted = true;
            if (!alive) {
                unsigned idx = base + __popc(need & ((1u << lane) - 1u));
                if (idx < nq) {
                    load_particle<Real, Multi>(P, P.pin, idx, p);
                    if (Adj) Gh = hist_weight(P, p);
                    alive = true;
                    s.state = 0;
                    s.nsteps = 0;
                    if (P.pin.st[idx] == 3) {   // resume a photon due to interact
                        const MedScalars<Real> &M = cmed<Real>(G.med[p.ir]);
                        s.state = 3;
                        s.medium = G.med[p.ir];
                        s.rhor = G.rhor[p.ir];
                        s.gle = dlog(p.E);
                        s.lgle = min(max((int)(M.ge1 * s.gle + M.ge0), 1), MXGE);
                        const Real *g = T.gtab + ((size_t)M.gtab_off + s.lgle - 1) * 8;
                        s.cohfac = g[7] * s.gle + g[6];
                    } else if (P.pin.st[idx]) {   // resume a parked photon
                        s.state = 1;
                        s.medium = G.med[p.ir];
                        s.rhor = G.rhor[p.ir];
                        s.gle = dlog(p.E);
                        s.dpmfp = P.pin.aux0[idx];
                    }
                }
            }
        }
        unsigned live = __ballot_sync(0xffffffffu, alive);
        if (!live) break;
        lanes += __popc(live);
        ++iters;
        // Interactions are sampled for several lanes at once: a lane whose
        // photon is due to interact waits until enough of the warp is due too
        // (or a bounded number of iterations has passed).
        {
            unsigned pend = __ballot_sync(0xffffffffu, alive && s.state == 3);
            bool batch = false;
            if (pend) {
                ++inter_wait;
                batch = __popc(pend) >= min(P.inter_batch_p, __popc(live)) || inter_wait > INTER_MAXWAIT;
            }
            if (batch) {
                inter_wait = 0;
                if (alive && s.state == 3) {
                // interaction
                p.rng.ahead(RNG_AHEAD);   // the batch's blocks, computed together
                ++ninter;
                if (Adj) gadd(P, ga, p.ir, Gh / s.rhor);
                const MedScalars<Real> &M = cmed<Real>(s.medium);
                const Real *g = T.gtab + ((size_t)M.gtab_off + s.lgle - 1) * 8;
                Real r37 = urand<Real>(p.rng);
                if (r37 <= 1 - s.cohfac) {   // Rayleigh (src/egsnrc.macros:1602-1613)
                    Real costhe, sinthe;
                    rayleigh(T, s.medium, p.E, s.gle, s.lgle, p.rng, costhe, sinthe, err);
                    Azim<Real> az = azimuth<Real>(p.rng, err);
                    Real a = p.u, b = p.v, c = p.w;
                    rotate(a, b, c, sinthe, costhe, az, p.u, p.v, p.w);
                    s.state = 0;
                    continue;
                }
                Real r36 = urand<Real>(p.rng);
                Real gbr1 = g[3] * s.gle + g[2];
                if (r36 <= gbr1 && p.E > 2 * rm) {
                    Real E2, u2, v2, w2;
                    int iq2;
                    pair(M, p, E2, iq2, u2, v2, w2, err);
                    Particle<Real> q = p;
                    q.E = E2; q.iq = iq2; q.u = u2; q.v = v2; q.w = w2;
                    q.rng.init(p.rng.seed, p.rng.hist, child_sid(p.rng.sid, p.rng.n, 0), 0u);
                    push_charged(P, P.ein, P.pout, p, acc, npush, edep_tot, err);
                    push_charged(P, P.ein, P.pout, q, acc, npush, edep_tot, err);
                    alive = false;
                    continue;
                }
                Real gbr2 = g[5] * s.gle + g[4];
                if (r36 < gbr2) {
                    Particle<Real> e = p;
                    Real edep = compton(T, M, p, e.u, e.v, e.w, e.E, err);
                    e.iq = -1;
                    e.rng.init(p.rng.seed, p.rng.hist, child_sid(p.rng.sid, p.rng.n, 0), 0u);
                    if (edep > 0) { deposit(P, acc, p.ir, p.rng.hist, edep * p.wt); edep_tot += (double)(edep * p.wt); }
                    push_charged(P, P.ein, P.pout, e, acc, npush, edep_tot, err);
                    s.state = 0;
                    continue;
                }
                Real edep = photo(T, M, p, s.gle, err);
                if (edep > 0) { deposit(P, acc, p.ir, p.rng.hist, edep * p.wt); edep_tot += (double)(edep * p.wt); }
                push_charged(P, P.ein, P.pout, p, acc, npush, edep_tot, err);
                alive = false;
                }
                continue;
            }
        }
        if (!alive || s.state == 3) continue;

        if (s.state == 0) {   // :PNEWENERGY:
            if (p.E <= T.pcut) {   // :PCUT-DISCARD:
                deposit(P, acc, p.ir, p.rng.hist, p.E * p.wt);
                edep_tot += (double)(p.E * p.wt);
                alive = false;
                continue;
            }
            s.medium = G.med[p.ir];
            s.rhor = G.rhor[p.ir];
            s.gle = dlog(p.E);
            Real r35 = urand<Real>(p.rng);
            s.dpmfp = -dlog(r35);
            s.state = 1;
        }
        if (s.state == 1) {   // :PNEWMEDIUM:
            const MedScalars<Real> &M = cmed<Real>(s.medium);
            s.lgle = min(max((int)(M.ge1 * s.gle + M.ge0), 1), MXGE);
            const Real *g = T.gtab + ((size_t)M.gtab_off + s.lgle - 1) * 8;
            s.gmfpr0 = g[1] * s.gle + g[0];
            s.cohfac = g[7] * s.gle + g[6];
            s.state = 2;
        }
        // :PTRANS: one voxel
        if (++s.nsteps > STEP_CAP) { err = 1; alive = false; continue; }
        Real gmfp = s.gmfpr0 / s.rhor * s.cohfac;
        Real ustep = gmfp * s.dpmfp;
        if (HFL) {
            ++nstep;
            if (hfl_dist_out(G, p) <= ustep) { esc_tot += (double)(p.E * p.wt); alive = false; continue; }
            p.x += p.u * ustep; p.y += p.v * ustep; p.z += p.w * ustep;
            s.dpmfp = 0;
            p.ir = hfl_locate(G, p.x, p.y, p.z);
            s.state = 3;
            continue;
        }
#pragma unroll 1
        for (int hop = 0;; ++hop) {
            if (hop) { gmfp = s.gmfpr0 / s.rhor * s.cohfac; ustep = gmfp * s.dpmfp; }
            int irnew = howfar(geom_of<Real, Multi>(P, p.pb), p.ir, p.x, p.y, p.z, p.u, p.v, p.w, ustep);
            ++nstep;
            if (Adj) gadd(P, ga, p.ir, -Gh * (ustep / gmfp) / s.rhor);
            p.x += p.u * ustep; p.y += p.v * ustep; p.z += p.w * ustep;
            s.dpmfp = dmax((Real)0, s.dpmfp - ustep / gmfp);
            if (irnew != p.ir) {
                p.ir = irnew;
                if (irnew < 0) { esc_tot += (double)(p.E * p.wt); alive = false; break; }
                int mnew = G.med[irnew];
                s.rhor = G.rhor[irnew];
                if (mnew != s.medium) { s.medium = mnew; s.state = 1; break; }
            }
            if (!(s.dpmfp > (Real)1e-8)) { s.state = 3; break; }
            if (hop + 1 >= PHOTON_HOPS || ++s.nsteps > STEP_CAP) break;
        }
    }
    acc_flush(P, acc);
    if (Adj) gflush(P, ga);
    // block-level counter reduction via warp shuffles
    for (int o = 16; o > 0; o >>= 1) {
        nstep += __shfl_down_sync(0xffffffffu, nstep, o);
        npush += __shfl_down_sync(0xffffffffu, npush, o);
        ninter += __shfl_down_sync(0xffffffffu, ninter, o);
        edep_tot += __shfl_down_sync(0xffffffffu, edep_tot, o);
        esc_tot += __shfl_down_sync(0xffffffffu, esc_tot, o);
    }
    if (lane == 0) {
        atomicAdd(P.counters + CNT_PLANES, lanes);
        atomicAdd(P.counters + CNT_PITER, iters);
        atomicAdd(P.counters + CNT_PSTEP, nstep);
        atomicAdd(P.counters + CNT_PUSH, npush);
        atomicAdd(P.counters + CNT_INTER, ninter);
        atomicAdd(P.energy + 0, edep_tot);
        atomicAdd(P.energy + 1, esc_tot);
    }
    if (err) atomicExch(P.error + 1, 1);
}

// ----------------------------------------------------------- electron ----
template <class Real>
struct ElecState {
    int state;            // 0 new electron, 1 new tstep, 2 ustep
    int medium, lelke, compute_tstep, nsteps;
    Real rhor, eke, elke, sig0, demfp;
    Real total_de, total_tstep;
};

// Electron-table row accessor: 16 coefficients per energy bin.
template <class Real>
struct ERow {
    const Real *r;
    int qel;
    __device__ Real sig(Real elke) const { return qel ? r[3] * elke + r[2] : r[1] * elke + r[0]; }
    __device__ Real dedx(Real elke) const { return qel ? r[7] * elke + r[6] : r[5] * elke + r[4]; }
    __device__ Real dedx1() const { return qel ? r[7] : r[5]; }
};

template <class Real>
__device__ inline const Real *erow(const Tables<Real> &T, const MedScalars<Real> &M, int lel) {
    return T.etab + ((size_t)M.etab_off + lel - 1) * 16;
}
template <class Real>
__device__ inline const Real *rrow(const Tables<Real> &T, const MedScalars<Real> &M, int lel) {
    return T.erange + ((size_t)M.etab_off + lel - 1) * 4;
}

// The residual-range and energy-loss macros take their arithmetic type C
// apart from the table type Real: the FP32 kernels run them in FP64 where a
// step ends near a voxel face or near the end of the range (see
// k_electron's `wide` steps), from the same FP32 table rows.
// $COMPUTE-DRANGE (src/egsnrc.macros:3214-3238)
template <class C, class Real>
__device__ inline C drange(const Tables<Real> &T, const MedScalars<Real> &M, int qel, C e1, C e2, int lel, C el1,
                           C el2) {
    const Real *r = erow(T, M, lel);
    C fedep = 1 - e2 / e1;
    C elktmp = (C)0.5 * (el1 + el2 + (C)0.25 * fedep * fedep * (1 + fedep * (1 + (C)0.875 * fedep)));
    C d0 = qel ? (C)r[6] : (C)r[4], d1 = qel ? (C)r[7] : (C)r[5];
    C dedxmid = 1 / (d1 * elktmp + d0);
    C aux = d1 * dedxmid;
    aux = aux * (1 + 2 * aux) * (fedep / (2 - fedep)) * (fedep / (2 - fedep)) / 6;
    return fedep * e1 * dedxmid * (1 + aux);
}
// $COMPUTE-ELOSS (:3290-3312)
template <class C, class Real>
__device__ inline C eloss(const Tables<Real> &T, const MedScalars<Real> &M, int qel, C step, C eke, C elke, int lel,
                          C rhof) {
    const Real *r = erow(T, M, lel);
    C d0 = qel ? (C)r[6] : (C)r[4], d1 = qel ? (C)r[7] : (C)r[5];
    C dedxmid = d1 * elke + d0;
    C aux = d1 / dedxmid;
    C de = dedxmid * step * rhof;
    C fedep = de / eke;
    return de * (1 - (C)0.5 * fedep * aux * (1 - (C)0.333333 * fedep * (aux - 1 - (C)0.25 * fedep * (2 - aux * (4 - aux)))));
}
// $COMPUTE-ELOSS-G (:3315-3351)
template <class C, class Real>
__device__ inline C eloss_g(const Tables<Real> &T, const MedScalars<Real> &M, int qel, C step, C eke, C elke, int lel,
                            C range, C rhof) {
    C tuss = range - (C)rrow(T, M, lel)[1 + qel] / rhof;
    if (tuss >= step) return eloss<C>(T, M, qel, step, eke, elke, lel, rhof);
    int lt = lel;
    tuss = (range - step) * rhof;
    if (tuss <= 0) return eke - (C)M.te * (C)0.99;
    while (lt > 1 && tuss < (C)rrow(T, M, lt)[1 + qel]) --lt;
    if (lt > M.meke - 1) lt = M.meke - 1;
    C elktmp = (lt + 1 - (C)M.eke0) / (C)M.eke1, eketmp = (C)rrow(T, M, lt + 1)[0];
    tuss = ((C)rrow(T, M, lt + 1)[1 + qel] - tuss) / rhof;
    C de = eloss<C>(T, M, qel, tuss, eketmp, elktmp, lt, rhof);
    return de + eke - eketmp;
}

// EGS_XYZGeometry::hownear in arithmetic type C from the kernel's FP32 or
// FP64 positions and planes.
template <class C, class Real>
__device__ inline C hownear_c(const Geom<Real> &G, int ireg, Real x, Real y, Real z) {
    const int loc = ireg - G.voff;
    int iz = fdiv(loc, G.mnxy, G.lnxy), ir = loc - iz * G.nxy, iy = fdiv(ir, G.mnx, G.lnx), ix = ir - iy * G.nx;
    C t = dmin((C)x - (C)G.xb[ix], (C)G.xb[ix + 1] - (C)x);
    t = dmin(t, dmin((C)y - (C)G.yb[iy], (C)G.yb[iy + 1] - (C)y));
    t = dmin(t, dmin((C)z - (C)G.zb[iz], (C)G.zb[iz + 1] - (C)z));
    return t;
}
// EGS_XYZGeometry::howfar (egs_nd_geometry.h:963-1104) with the face
// distances in arithmetic type C; t is compared and returned in C.
template <class C, class Real>
__device__ inline int howfar_c(const Geom<Real> &G, int ireg, Real x, Real y, Real z, Real u, Real v, Real w, C &t,
                               int &axis) {
    const int loc = ireg - G.voff;
    int iz = fdiv(loc, G.mnxy, G.lnxy), ir = loc - iz * G.nxy, iy = fdiv(ir, G.mnx, G.lnx), ix = ir - iy * G.nx;
    int inew = ireg;
    const C bt = (C)G.bt, hbt = (C)G.hbt;
    if (u > 0) {
        C d = ((C)G.xb[ix + 1] - (C)x) / (C)u;
        if (d <= t) { t = (d <= bt) ? hbt : d; inew = (ix + 1 < G.nx) ? ireg + 1 : -1; axis = 0; }
    } else if (u < 0) {
        C d = ((C)G.xb[ix] - (C)x) / (C)u;
        if (d <= t) { t = (d <= bt) ? hbt : d; inew = (ix - 1 >= 0) ? ireg - 1 : -1; axis = 0; }
    }
    if (v > 0) {
        C d = ((C)G.yb[iy + 1] - (C)y) / (C)v;
        if (d <= t) { t = (d <= bt) ? hbt : d; inew = (iy + 1 < G.ny) ? ireg + G.nx : -1; axis = 1; }
    } else if (v < 0) {
        C d = ((C)G.yb[iy] - (C)y) / (C)v;
        if (d <= t) { t = (d <= bt) ? hbt : d; inew = (iy - 1 >= 0) ? ireg - G.nx : -1; axis = 1; }
    }
    if (w > 0) {
        C d = ((C)G.zb[iz + 1] - (C)z) / (C)w;
        if (d <= t) { t = (d <= bt) ? hbt : d; inew = (iz + 1 < G.nz) ? ireg + G.nxy : -1; axis = 2; }
    } else if (w < 0) {
        C d = ((C)G.zb[iz] - (C)z) / (C)w;
        if (d <= t) { t = (d <= bt) ? hbt : d; inew = (iz - 1 >= 0) ? ireg - G.nxy : -1; axis = 2; }
    }
    return inew;
}

// The FP64 pieces of a `wide` step of the FP32 electron kernel, kept out of
// line so that the FP32 step does not carry their registers.
template <class Real>
__device__ __noinline__ double wide_range(const Tables<Real> &T, const MedScalars<Real> &M, int qel, Real eke,
                                          Real elke, int lelke, Real rhof) {
    const Real *rr = rrow(T, M, lelke);
    const double r0 = drange<double>(T, M, qel, (double)eke, (double)rr[0], lelke, (double)elke,
                                     ((double)lelke - (double)M.eke0) / (double)M.eke1);
    return (r0 + (double)rr[1 + qel]) / (double)rhof;
}
template <class Real>
__device__ __noinline__ Real wide_hownear(const Geom<Real> &G, int ireg, Real x, Real y, Real z) {
    return (Real)hownear_c<double>(G, ireg, x, y, z);
}
template <class Real>
__device__ __noinline__ int wide_howfar(const Geom<Real> &G, int ireg, Real x, Real y, Real z, Real u, Real v, Real w,
                                        Real &t, int &axis) {
    double tw = t;
    const int inew = howfar_c<double>(G, ireg, x, y, z, u, v, w, tw, axis);
    t = (Real)tw;
    return inew;
}
template <class Real>
__device__ __noinline__ Real wide_eloss(const Tables<Real> &T, const MedScalars<Real> &M, int qel, double step, Real eke,
                                        Real elke, int lelke, double range, Real rhof) {
    return (Real)eloss_g<double>(T, M, qel, step, (double)eke, (double)elke, lelke, range, (double)rhof);
}

// Adj: adjoint replay of the continuous energy loss (see EList).
// HFL: HOWFARLESS transport with hinge dose deposition (hfl_hinge).
// PI: PRESTA-I boundary crossing instead of EXACT (src/egsnrc.mortran:1247-1345):
// every step within tperp is a PRESTA-II step; a step that reaches past the
// nearest boundary is shortened by the average path-length correction
// ($SET-USTEP), corrected back if howfar cuts it ($SET-TVSTEP), and deflected
// once at its end by mscat.  Its own instantiation, so that the EXACT kernels
// carry none of this code.
// SPL: the precision split of the FP32 kernel (egsgpu_config.fp64_near_faces),
// its own instantiation so that the default FP32 step carries none of it.
template <class Real, bool Multi, bool Adj = false, bool HFL = false, bool PI = false, bool SPL = false>
__global__ void __launch_bounds__(MAX_BLOCK, sizeof(Real) == 4 && !Adj ? 6 : 1) k_electron(Params<Real> P) {
    const Tables<Real> &T = P.T;
    const Geom<Real> &G = P.G;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned nq = *P.ein.count < P.ein.capacity ? *P.ein.count : P.ein.capacity;
    if (threadIdx.x == 0 && blockIdx.x == 0) atomicMax(P.peak, *P.ein.count);
    Particle<Real> p;
    ElecState<Real> s;
    Real edep_part = 0;   // continuous-loss deposits of the current particle
    // EGSnrc's own stack discipline for the charged secondaries of Moller and
    // Bhabha events: the primary is suspended on a small per-thread LIFO (in
    // local memory) and the secondary is followed first; a full stack spills
    // to the next electron queue.
    Particle<Real> lstack[LSTACK];
    int sp = 0;
    Acc<Real> acc{-1, 0u, (Real)0};
    EList<Real> el;
    el.n = 0;
    // adjoint: the voxel-visit lists of suspended particles; a secondary
    // starts from a copy of its parent's list (chords to its creation point,
    // coefficients zero), so that its crossings also see the parent's path
    EList<Real> elstack[Adj ? LSTACK : 1];
    bool alive = false, exhausted = false;
    unsigned long long nstep = 0, npush = 0, ninter = 0, lanes = 0, iters = 0, nwide = 0;
    constexpr bool SPLIT = sizeof(Real) == 4 && !HFL && SPL;   // the FP32 kernel's FP64 steps (`wide`)
    int inter_wait = 0;   // warp-uniform iterations since the first lane became due
    double edep_tot = 0, esc_tot = 0;
    int err = 0;
    const Real rm = (Real)RM;
    const bool requeue = P.requeue_lanes > 0 && nq >= REQUEUE_MIN;
    while (true) {
        if (!alive && sp > 0) {   // resume a suspended particle
            p = lstack[--sp];
            if (Adj) el = elstack[sp];
            alive = true;
            s.state = 0;
            s.nsteps = 0;
            s.medium = G.med[p.ir];
            s.rhor = G.rhor[p.ir];
        }
        if (exhausted && requeue) {
            unsigned busy = __ballot_sync(0xffffffffu, alive);
            if (__popc(busy) <= P.requeue_lanes) {   // park the survivors and retire the warp
                while (sp > 0) q_push(P, P.eout, lstack[--sp], npush);
                if (alive) {
                    unsigned i = q_slot(P, P.eout);
                    if (i != ~0u) {
                        q_store(P.eout, i, p);
                        if (s.state == 1) P.eout.st[i] = 1;
                        else if (s.state == 3) P.eout.st[i] = 8;
                        else if (s.state == 2) {
                            P.eout.st[i] = (uint8_t)(2 | (s.compute_tstep ? 4 : 0));
                            P.eout.aux0[i] = s.demfp; P.eout.aux1[i] = s.total_de;
                            P.eout.aux2[i] = s.total_tstep; P.eout.aux3[i] = s.sig0;
                        }
                    }
                }
                break;
            }
        }
        unsigned need = __ballot_sync(0xffffffffu, !alive);
        if (need && !exhausted) {
            unsigned base = 0;
            if (lane == (unsigned)(__ffs(need) - 1)) base = atomicAdd(P.ein.count + 1, (unsigned)__popc(need));
            base = __shfl_sync(0xffffffffu, base, __ffs(need) - 1);
            if (base >= nq) exhausted = true;
            if (!alive) {
                edep_tot += (double)edep_part;
                edep_part = 0;
                unsigned idx = base + __popc(need & ((1u << lane) - 1u));
                if (idx < nq) {
                    load_particle<Real, Multi>(P, P.ein, idx, p);
                    if (Adj) el.n = 0;
                    alive = true;
                    s.state = 0;
                    s.nsteps = 0;
                    s.medium = G.med[p.ir];
                    s.rhor = G.rhor[p.ir];
                    uint8_t st = P.ein.st[idx];
                    if (st == 1) s.state = 1;
                    else if (st == 8) {   // resume a particle due to interact
                        const MedScalars<Real> &M = cmed<Real>(s.medium);
                        s.state = 3;
                        s.eke = p.E - (Real)RM;
                        s.elke = dlog(s.eke);
                        s.lelke = min(max((int)(M.eke1 * s.elke + M.eke0), 1), M.meke);
                    }
                    else if (st & 2) {   // resume a parked condensed-history sequence
                        const MedScalars<Real> &M = cmed<Real>(s.medium);
                        s.state = 2;
                        s.compute_tstep = (st & 4) ? 1 : 0;
                        s.demfp = P.ein.aux0[idx]; s.total_de = P.ein.aux1[idx];
                        s.total_tstep = P.ein.aux2[idx]; s.sig0 = P.ein.aux3[idx];
                        s.eke = p.E - (Real)RM;
                        s.elke = dlog(s.eke);
                        s.lelke = min(max((int)(M.eke1 * s.elke + M.eke0), 1), M.meke);
                    }
                }
            }
        }
        unsigned live = __ballot_sync(0xffffffffu, alive);
        if (!live) break;
        lanes += __popc(live);
        ++iters;
        // the random-number blocks of the coming step, computed by the warp's
        // live lanes together (Rng::ahead)
        if (alive) p.rng.ahead(RNG_AHEAD);
        // Discrete interactions are sampled for several lanes at once (see the
        // photon kernel).
        {
            unsigned pend = __ballot_sync(0xffffffffu, alive && s.state == 3);
            bool batch = false;
            if (pend) {
                ++inter_wait;
                batch = __popc(pend) >= min(P.inter_batch, __popc(live)) || inter_wait > INTER_MAXWAIT;
            }
            if (batch) {
                inter_wait = 0;
                if (alive && s.state == 3) {
                const int qel = (1 + p.iq) / 2;
                const MedScalars<Real> &M2 = cmed<Real>(s.medium);
                ERow<Real> ef{erow(T, M2, s.lelke), qel};
                    // discrete interaction
                    ++ninter;
                    const Real *rw = ef.r;
                    bool brems = false;
                    if (p.iq < 0) {
                        Real ebr1 = rw[9] * s.elke + rw[8];
                        Real r24 = urand<Real>(p.rng);
                        brems = r24 <= ebr1;
                        if (!brems && p.E <= M2.thmoll) {
                            if (ebr1 <= 0) { s.state = 0; continue; }
                            brems = true;
                        }
                        if (!brems) {   // MOLLER (src/egsnrc.mortran:2599-2746)
                            Real peie = p.E, ekin = peie - rm;
                            if (ekin <= 2 * M2.te) { s.state = 0; continue; }
                            Real t0 = ekin / rm, e0 = t0 + 1, extrae = peie - M2.thmoll, e02 = e0 * e0;
                            Real g2 = t0 * t0 / e02, g3 = (2 * t0 + 1) / e02, gmax = 1 + (Real)1.25 * g2, br, rejf4, r28;
                            int it = 0;
                            do {
                                float2 q = urand2(p.rng);
                                Real r27 = (Real)q.x;
                                br = M2.te / (ekin - extrae * r27);
                                Real rr2 = br / (1 - br);
                                r28 = (Real)q.y;
                                rejf4 = 1 + g2 * br * br + rr2 * (rr2 - g3);
                                r28 = gmax * r28;
                                if (++it > LOOP_CAP) { err = 1; break; }
                            } while (!(r28 <= rejf4));
                            Real pekse2 = br * ekin, pese1 = peie - pekse2, pese2 = pekse2 + rm;
                            Real h1 = (peie + rm) / ekin;
                            Real dcosth = h1 * (pese1 - rm) / (pese1 + rm);
                            Real sinthe = dsqrt(dmax((Real)0, 1 - dcosth)), costhe = dsqrt(dmin((Real)1, dcosth));
                            Azim<Real> az = azimuth<Real>(p.rng, err);
                            Real a = p.u, b = p.v, c = p.w;
                            rotate(a, b, c, sinthe, costhe, az, p.u, p.v, p.w);
                            p.E = pese1;
                            Particle<Real> d = p;
                            d.rng.init(p.rng.seed, p.rng.hist, child_sid(p.rng.sid, p.rng.n, 0), 0u);
                            dcosth = h1 * (pese2 - rm) / (pese2 + rm);
                            sinthe = -dsqrt(dmax((Real)0, 1 - dcosth));
                            costhe = dsqrt(dmin((Real)1, dcosth));
                            rotate(a, b, c, sinthe, costhe, az, d.u, d.v, d.w);
                            d.E = pese2; d.iq = -1;
                            if (d.E > T.ecut && sp < LSTACK) {
                                lstack[sp] = p;
                                if (Adj) {
                                    elstack[sp] = el;
                                    for (int i = 0; i < el.n; ++i) el.k[i] = 0;
                                }
                                ++sp;
                                p = d;
                            }
                            else push_charged(P, P.eout, P.pout, d, acc, npush, edep_tot, err);
                            s.state = 0;
                            continue;
                        }
                    } else {
                        Real pbr1 = rw[11] * s.elke + rw[10];
                        Real r25 = urand<Real>(p.rng);
                        if (r25 < pbr1) brems = true;
                        else {
                            Real pbr2 = rw[13] * s.elke + rw[12];
                            if (r25 < pbr2) {   // BHABHA (src/egsnrc.mortran:229-307)
                                Real peip = p.E, ekin = peip - rm, t0 = ekin / rm, e0 = t0 + 1;
                                Real yy = 1 / (t0 + 2), e02 = e0 * e0, beta2b = (e02 - 1) / e02;
                                Real ep0 = M2.te / ekin, ep0c = 1 - ep0, y2 = yy * yy, yp = 1 - 2 * yy, yp2 = yp * yp;
                                Real b4 = yp2 * yp, b3 = b4 + yp2, b2 = yp * (3 + y2), b1 = 2 - y2, br, rejf2, r04;
                                int it = 0;
                                do {
                                    float2 q = urand2(p.rng);
                                    Real r03 = (Real)q.x;
                                    br = ep0 / (1 - ep0c * r03);
                                    r04 = (Real)q.y;
                                    rejf2 = (1 - beta2b * br * (b1 - br * (b2 - br * (b3 - br * b4))));
                                    if (++it > LOOP_CAP) { err = 1; break; }
                                } while (!(r04 <= rejf2));
                                int iq_np = 1, iq_new = -1;
                                if (!(br < (Real)0.5)) { iq_np = -1; iq_new = 1; br = 1 - br; }
                                br = dmax(br, (Real)0);
                                Real pekse2 = br * ekin, pese1 = peip - pekse2, pese2 = pekse2 + rm;
                                Real h1 = (peip + rm) / ekin;
                                Real dcosth = dmin((Real)1, h1 * (pese1 - rm) / (pese1 + rm));
                                Real sinthe = dsqrt(dmax((Real)0, 1 - dcosth)), costhe = dsqrt(dcosth);
                                Azim<Real> az = azimuth<Real>(p.rng, err);
                                Real a = p.u, b = p.v, c = p.w;
                                rotate(a, b, c, sinthe, costhe, az, p.u, p.v, p.w);
                                p.E = pese1; p.iq = iq_np;
                                Particle<Real> d = p;
                                d.rng.init(p.rng.seed, p.rng.hist, child_sid(p.rng.sid, p.rng.n, 0), 0u);
                                dcosth = h1 * (pese2 - rm) / (pese2 + rm);
                                sinthe = -dsqrt(dmax((Real)0, 1 - dcosth));
                                costhe = dsqrt(dmin((Real)1, dcosth));
                                rotate(a, b, c, sinthe, costhe, az, d.u, d.v, d.w);
                                d.E = pese2; d.iq = iq_new;
                                if (d.E > T.ecut && sp < LSTACK) {
                                lstack[sp] = p;
                                if (Adj) {
                                    elstack[sp] = el;
                                    for (int i = 0; i < el.n; ++i) el.k[i] = 0;
                                }
                                ++sp;
                                p = d;
                            }
                                else push_charged(P, P.eout, P.pout, d, acc, npush, edep_tot, err);
                                s.state = 0;
                                continue;
                            }
                            // ANNIH in flight (src/egsnrc.mortran:70-182)
                            Real pavip = p.E + rm, avip = pavip, a = avip / rm, gg = a - 1, tt = gg - 1;
                            Real pp = dsqrt(a * tt), pot = pp / tt, ep0 = 1 / (a + pp), wsamp = dlog((1 - ep0) / ep0);
                            Real aa = p.u, bb = p.v, cc = p.w, ep, r02, rejf;
                            int it = 0;
                            do {
                                float2 q = urand2(p.rng);
                                Real r01 = (Real)q.x;
                                ep = ep0 * dexp(r01 * wsamp);
                                r02 = (Real)q.y;
                                rejf = 1 - (ep * a - 1) * (ep * a - 1) / (ep * (a * a - 2));
                                if (++it > LOOP_CAP) { err = 1; break; }
                            } while (!(r02 <= rejf));
                            Real esg1 = avip * ep;
                            Real costhe = dmax((Real)-1, dmin((Real)1, (esg1 - rm) * pot / esg1));
                            Real sinthe = dsqrt(1 - costhe * costhe);
                            Azim<Real> az = azimuth<Real>(p.rng, err);
                            Particle<Real> g1 = p, g2 = p;
                            g1.E = esg1; g1.iq = 0;
                            rotate(aa, bb, cc, sinthe, costhe, az, g1.u, g1.v, g1.w);
                            g2.rng.init(p.rng.seed, p.rng.hist, child_sid(p.rng.sid, p.rng.n, 0), 0u);
                            Real esg2 = pavip - esg1;
                            g2.E = esg2; g2.iq = 0;
                            costhe = dmax((Real)-1, dmin((Real)1, (esg2 - rm) * pot / esg2));
                            sinthe = -dsqrt(1 - costhe * costhe);
                            rotate(aa, bb, cc, sinthe, costhe, az, g2.u, g2.v, g2.w);
                            q_push(P, P.pout, g1, npush);
                            q_push(P, P.pout, g2, npush);
                            if (Adj) elist_flush(P, el);
                            alive = false;
                            continue;
                        }
                    }
                    // BREMS, BH cross section with KM angles (src/egsnrc.mortran:312-524)
                    {
                        Real peie = p.E, ekin = peie - rm, brmin = M2.ap / ekin, waux = s.elke - M2.log_ap;
                        int l = (peie < 50) ? 0 : 2, l1 = l + 1;
                        Real a = p.u, b = p.v, c = p.w, sinpsi = a * a + b * b, sindel = 0, cosdel = 0;
                        if (sinpsi > (Real)1e-20) { sinpsi = dsqrt(sinpsi); sindel = b / sinpsi; cosdel = a / sinpsi; }
                        Real tteie = peie / rm;
                        Real beta = dsqrt((tteie - 1) * (tteie + 1)) / tteie;
                        Real y2max = 2 * beta * (1 + beta) * tteie * tteie, y2maxi = 1 / y2max;
                        Real z2maxi = dsqrt(y2max + 1);
                        Real esg, ese, r07, rejf;
                        int it = 0;
                        do {
                            float2 q = urand2(p.rng);
                            Real r06 = (Real)q.x;
                            r07 = (Real)q.y;
                            Real br = brmin * dexp(r06 * waux);
                            esg = ekin * br;
                            ese = peie - esg;
                            Real delta = esg / peie / ese * M2.delcm, aux = ese / peie, phi1, phi2;
                            if (delta < 1) {
                                phi1 = M2.dl[0][l] + delta * (M2.dl[1][l] + delta * M2.dl[2][l]);
                                phi2 = M2.dl[0][l1] + delta * (M2.dl[1][l1] + delta * M2.dl[2][l1]);
                            } else {
                                phi1 = M2.dl[3][l] + M2.dl[4][l] * dlog(delta + M2.dl[5][l]);
                                phi2 = phi1;
                            }
                            rejf = (1 + aux * aux) * phi1 - 2 * aux * phi2 / 3;
                            if (++it > LOOP_CAP) { err = 1; break; }
                        } while (!(r07 < rejf));
                        Real ttese = ese / rm, esedei = ttese / tteie, rjarg1 = 1 + esedei * esedei;
                        Real rjarg2 = rjarg1 + 2 * esedei;
                        Real aux = 2 * ese * tteie / esg;
                        aux = aux * aux;
                        Real aux1 = aux * M2.zbrang, rjarg3;
                        if (aux1 > 10) rjarg3 = M2.lzbrang + (1 - aux1) / (aux1 * aux1);
                        else rjarg3 = dlog(aux / (1 + aux1));
                        Real rejmax = rjarg1 * rjarg3 - rjarg2, y2tst, rtest;
                        it = 0;
                        while (true) {
                            float2 q = urand2(p.rng);
                            y2tst = (Real)q.x;
                            rtest = (Real)q.y;
                            Real aux3 = z2maxi / (y2tst + (1 - y2tst) * z2maxi);
                            rtest = rtest * aux3 * rejmax;
                            y2tst = aux3 * aux3 - 1;
                            Real a34 = aux3 * aux3 * aux3 * aux3;
                            Real y2tst1 = esedei * y2tst / a34;
                            Real aux4 = 16 * y2tst1 - rjarg2, aux5 = rjarg1 - 4 * y2tst1;
                            if (rtest < aux4 + aux5 * rjarg3) break;
                            Real aux2 = dlog(aux / (1 + aux1 / a34));
                            Real rejtst = aux4 + aux5 * aux2;
                            if (rtest < rejtst) break;
                            if (++it > LOOP_CAP) { err = 1; break; }
                        }
                        Real costhe = 1 - 2 * y2tst * y2maxi;
                        Real sinthe = dsqrt(dmax((1 - costhe) * (1 + costhe), (Real)0));
                        Azim<Real> az = azimuth<Real>(p.rng, err);
                        Particle<Real> gph = p;
                        gph.rng.init(p.rng.seed, p.rng.hist, child_sid(p.rng.sid, p.rng.n, 0), 0u);
                        gph.E = esg; gph.iq = 0;
                        if (sinpsi >= (Real)1e-10) {
                            Real us = sinthe * az.c, vs = sinthe * az.s;
                            gph.u = c * cosdel * us - sindel * vs + a * costhe;
                            gph.v = c * sindel * us + cosdel * vs + b * costhe;
                            gph.w = c * costhe - sinpsi * us;
                        } else { gph.u = sinthe * az.c; gph.v = sinthe * az.s; gph.w = c * costhe; }
                        q_push(P, P.pout, gph, npush);
                        p.E = ese;
                        s.state = 0;
                        continue;
                    }
                }
                continue;
            }
        }
        if (!alive || s.state == 3) continue;

        const int qel = (1 + p.iq) / 2;
        bool ecut_discard = false;
        if (++s.nsteps > STEP_CAP) { err = 1; alive = false; continue; }
        if (s.state == 0) {   // :NEWELECTRON:
            if (p.E <= T.ecut) ecut_discard = true;
            else s.state = 1;
        }
        if (!ecut_discard) {
            if (s.state == 1) {   // :TSTEP:
                const MedScalars<Real> &M = cmed<Real>(s.medium);
                s.compute_tstep = 1;
                s.eke = p.E - rm;
                Real r = urand<Real>(p.rng);
                s.demfp = dmax(-dlog(r), (Real)1e-8);
                s.elke = dlog(s.eke);
                s.lelke = min(max((int)(M.eke1 * s.elke + M.eke0), 1), M.meke);
                ERow<Real> er{erow(T, M, s.lelke), qel};
                if (qel ? M.sig_mono_p : M.sig_mono_e) s.sig0 = er.sig(s.elke) / er.dedx(s.elke);
                else s.sig0 = qel ? M.psig_e : M.esig_e;
                s.state = 2;
            }
            // :USTEP: one condensed-history step
            const MedScalars<Real> &M = cmed<Real>(s.medium);
            Real rhof = s.rhor, sig = s.sig0;
            Real tstep;
            const Real *rr = rrow(T, M, s.lelke);
            // range from the current energy to the lower edge of its bin
            // ($COMPUTE-DRANGE): serves both tstep and the residual range
            const Real r0 = drange<Real>(T, M, qel, (Real)s.eke, rr[0], s.lelke, (Real)s.elke,
                                   (s.lelke - (Real)M.eke0) / (Real)M.eke1);
            if (sig <= 0) { tstep = (Real)1e8; s.sig0 = (Real)1e-15; }
            else {
                if (s.compute_tstep) {
                    s.total_de = (Real)s.demfp / (Real)sig;
                    Real eke = s.eke, elke = s.elke, ekef = eke - s.total_de;
                    if (ekef <= M.E_array0) tstep = (Real)1e8;
                    else {
                        Real elkef = dlog(ekef);
                        int lelkef = min(max((int)((Real)M.eke1 * elkef + (Real)M.eke0), 1), s.lelke);
                        if (lelkef == s.lelke) tstep = drange<Real>(T, M, qel, eke, ekef, s.lelke, elke, elkef);
                        else {
                            const Real *rf = rrow(T, M, lelkef + 1);
                            Real ekei = rf[0], elkei = (lelkef + 1 - (Real)M.eke0) / (Real)M.eke1;
                            tstep = drange<Real>(T, M, qel, ekei, ekef, lelkef, elkei, elkef);
                            tstep = tstep + r0 + rr[1 + qel] - rf[1 + qel];
                        }
                    }
                    s.total_tstep = tstep;
                    s.compute_tstep = 0;
                }
                tstep = s.total_tstep / (Real)rhof;
            }
            ERow<Real> er{erow(T, M, s.lelke), qel};
            const Real *row = er.r;
            Real dedx0 = er.dedx(s.elke), dedx = rhof * dedx0;
            Real tmxs = (row[15] * s.elke + row[14]) / rhof;
            Real range = (r0 + rr[1 + qel]) / (Real)rhof;
            tmxs = dmin(tmxs, T.smaxir);
            Real tustep = (Real)dmin(tstep, dmin((Real)tmxs, range));
            const Geom<Real> &GP = geom_of<Real, Multi>(P, p.pb);
            Real tperp = HFL ? hfl_hownear(GP, p) : hownear(GP, p.ir, p.x, p.y, p.z);
            Real blccl = rhof * M.blcc;
            Real p2 = s.eke * (s.eke + 2 * rm), beta2 = p2 / (p2 + rm * rm);
            Real ssmfp = beta2 / blccl, skindepth = T.skindepth * ssmfp;
            // Precision split of the FP32 kernels (egsgpu_config.fp64_near_faces):
            // a step that starts within NEAR_FACE of a voxel face, or one that
            // may reach the end of the range, is `wide`: its distance to the
            // nearest face, its howfar distances, its residual range and its
            // energy loss are computed in FP64 from the FP32 particle and table
            // values.  Everything else stays FP32; the FP64 build is FP64
            // throughout.
            const bool wide = SPLIT && (tperp < (Real)NEAR_FACE || range <= dmin(tstep, tmxs));
            double range_w = 0;
            if (wide) {
                tperp = wide_hownear(GP, p.ir, p.x, p.y, p.z);
                range_w = wide_range(T, M, qel, (Real)s.eke, (Real)s.elke, s.lelke, (Real)rhof);
                ++nwide;
            }
            tustep = dmin(tustep, dmax(tperp, skindepth));
            bool callhowfar, dosingle = false, callmsdist, domultiple = false;
            Real ustep, uf, vf, wf, xf, yf, zf;
            Real de = 0;
            // PRESTA-I: the multiple-scattering parameters of the step
            // ($CALCULATE-XI, src/egsnrc.macros:1323-1348; spin effects off)
            Real ms_beta2 = 0, ms_chia2 = 0, ms_xi = 0;
            auto calculate_xi = [&](Real ekems, Real len) {
                const Real pq2 = ekems * (ekems + 2 * rm), xccl = rhof * M.xcc;
                ms_beta2 = pq2 / (pq2 + rm * rm);
                ms_chia2 = xccl / (4 * blccl * pq2);
                ms_xi = (Real)0.5 * xccl / pq2 / ms_beta2 * len;
                ms_xi = ms_xi * (dlog(1 + 1 / ms_chia2) - 1 / (1 + ms_chia2));
            };
            ++nstep;
            if (tustep <= tperp && (PI || tustep > skindepth)) {
                callhowfar = false;
                callmsdist = true;
                ustep = tustep;
            } else if (PI) {   // $SET-USTEP (src/egsnrc.macros:1308-1321)
                callmsdist = false;
                domultiple = true;
                calculate_xi(s.eke - (Real)0.5 * tustep * dedx, tustep);
                ustep = ms_xi < (Real)0.1 ? tustep * (1 - ms_xi * ((Real)0.5 - ms_xi * (Real)0.166667))
                                          : tustep * (1 - dexp(-ms_xi)) / ms_xi;
                callhowfar = !(ustep < tperp);
            } else {
                callmsdist = false;
                Real rnnoss = urand<Real>(p.rng);
                if (rnnoss < (Real)1e-30) rnnoss = (Real)1e-30;
                Real lambda = -dlog(1 - rnnoss);
                Real g1 = s.eke / rm + 1;
                Real lambda_max = (Real)0.5 * blccl * rm / dedx * g1 * g1 * g1;
                if (lambda >= 0 && lambda_max > 0) {
                    Real tuss = (lambda < lambda_max) ? lambda * ssmfp * (1 - (Real)0.5 * lambda / lambda_max)
                                                       : (Real)0.5 * lambda * ssmfp;
                    if (tuss < tustep) { tustep = tuss; dosingle = true; }
                } else {
                    err = 1;
                    alive = false;
                    continue;
                }
                ustep = tustep;
                callhowfar = !(ustep < tperp);
            }
            const Real ustep0 = ustep;
            int irold = p.ir, irnew = p.ir, axis = -1;
            if (callhowfar) {
                if (HFL) irnew = hfl_howfar(GP, p, ustep);
                else if (wide) irnew = wide_howfar(GP, p.ir, p.x, p.y, p.z, p.u, p.v, p.w, ustep, axis);
                else irnew = howfar(GP, p.ir, p.x, p.y, p.z, p.u, p.v, p.w, ustep, axis);
            }
            if (Adj && irnew != irold && axis >= 0) {   // the step ends on a voxel face
                const Real ua = axis == 0 ? p.u : (axis == 1 ? p.v : p.w);
                const Real wa = (Real)P.wvox[irold], wb = irnew >= 0 ? (Real)P.wvox[irnew] : (Real)0;
                elist_step(P, el, irold, p.u * ustep, p.v * ustep, p.w * ustep);
                elist_cross(el, axis, ua, (wa - wb) * dedx);
            }
            if (ustep <= 0) ustep = 0;
            if (ustep == 0) {
                if (irnew != irold) {
                    p.ir = irnew;
                    if (irnew < 0) {
                        esc_tot += (double)((p.iq < 0 ? p.E - rm : p.E + rm) * p.wt);
                        if (Adj) elist_flush(P, el);
                        alive = false;
                        continue;
                    }
                    s.medium = G.med[irnew];
                    s.rhor = G.rhor[irnew];
                }
                if (p.E <= T.ecut) ecut_discard = true;
                else { s.state = 1; continue; }
            }
            if (!ecut_discard) {
                Real vstep = ustep, tvstep = callhowfar ? vstep : tustep;
                if (PI && callhowfar) {   // $SET-TVSTEP (src/egsnrc.macros:1350-1392)
                    if (vstep < ustep0) {
                        calculate_xi(s.eke - (Real)0.5 * tustep * vstep / ustep0 * dedx, vstep);
                        if (ms_xi < (Real)0.1) tvstep = vstep * (1 + ms_xi * ((Real)0.5 + ms_xi * (Real)0.333333));
                        else if (ms_xi < (Real)0.999999) tvstep = -vstep * dlog(1 - ms_xi) / ms_xi;
                        else { err = 1; alive = false; continue; }
                    } else tvstep = tustep;
                }
                if (!PI && callhowfar && tvstep != tustep) dosingle = false;
                if (wide) {   // a step limited by the range ends it exactly, as in FP64
                    const double tvw = (tvstep == range) ? range_w : (double)tvstep;
                    de = wide_eloss(T, M, qel, tvw, (Real)s.eke, (Real)s.elke, s.lelke, range_w, (Real)rhof);
                } else {
                    de = eloss_g<Real>(T, M, qel, (Real)tvstep, (Real)s.eke, (Real)s.elke, s.lelke, range, (Real)rhof);
                }
                if (callmsdist) msdist_pII(T, M, p, s.eke, (Real)de, tustep, rhof, uf, vf, wf, xf, yf, zf, err);
                Real edep = (Real)de, ekef = s.eke - edep;
                if (!callmsdist) {
                    xf = p.x + p.u * vstep; yf = p.y + p.v * vstep; zf = p.z + p.w * vstep;
                    if (dosingle) {   // sscat (src/egsnrc.mortran:3226-3262)
                        Real ekems = dmax(ekef, T.ecut - rm);
                        Real pp2 = ekems * (ekems + 2 * rm);
                        Real chia2 = M.xcc / (4 * M.blcc * pp2);
                        Real xi = urand<Real>(p.rng);
                        xi = 2 * chia2 * xi / (1 - xi + chia2);
                        Real costhe = 1 - xi, sinthe = dsqrt(xi * (2 - xi));
                        Azim<Real> az = azimuth<Real>(p.rng, err);
                        rotate(p.u, p.v, p.w, sinthe, costhe, az, uf, vf, wf);
                    } else if (PI && domultiple) {   // src/egsnrc.mortran:1480-1496, 1561-1567
                        const Real lambda = blccl * tvstep / ms_beta2 / (1 + ms_chia2);
                        MsState<Real> st;
                        st.find_index = true; st.i = 0; st.j = 0; st.omega2 = 0;
                        Real costhe, sinthe;
                        mscat(T, p.rng, lambda, ms_chia2, ms_xi, st, costhe, sinthe, err);
                        Azim<Real> az = azimuth<Real>(p.rng, err);
                        rotate(p.u, p.v, p.w, sinthe, costhe, az, uf, vf, wf);
                    } else { uf = p.u; vf = p.v; wf = p.w; }
                }
                if (HFL) {
                    const Real xi0[3] = {p.x, p.y, p.z}, ui0[3] = {p.u, p.v, p.w};
                    p.x = xf; p.y = yf; p.z = zf; p.u = uf; p.v = vf; p.w = wf;
                    Real lost;
                    int iend = hfl_hinge(P, acc, GP, p, xi0, ui0, (Real)tvstep, callmsdist, edep, lost, err);
                    if (iend < 0) {   // the straight segments left the phantom: the particle is gone
                        Real e = p.E - edep;
                        edep_part += (edep - lost) * p.wt;
                        esc_tot += (double)((lost + (p.iq < 0 ? e - rm : e + rm)) * p.wt);
                        alive = false;
                        continue;
                    }
                    if (irnew >= 0) { p.ir = iend; irold = irnew = iend; }
                } else
                deposit(P, acc, p.ir, p.rng.hist, edep * p.wt);   // AUSGAB(0)
                if (Adj && !(irnew != irold && axis >= 0))   // steps inside the voxel (crossings above)
                    elist_step(P, el, p.ir, xf - p.x, yf - p.y, zf - p.z);
                edep_part += edep * p.wt;
                p.x = xf; p.y = yf; p.z = zf; p.u = uf; p.v = vf; p.w = wf;
                p.E = p.E - edep;
                if (irnew == p.ir && p.E <= T.ecut) ecut_discard = true;
                else {
                    int medold = s.medium;
                    s.eke = p.E - rm;
                    s.elke = dlog(s.eke);
                    s.lelke = min(max((int)(M.eke1 * s.elke + M.eke0), 1), M.meke);
                    if (irnew != irold) {
                        p.ir = irnew;
                        if (irnew < 0) {
                            esc_tot += (double)((p.iq < 0 ? p.E - rm : p.E + rm) * p.wt);
                            if (Adj) elist_flush(P, el);
                            alive = false;
                            continue;
                        }
                        s.medium = G.med[irnew];
                        s.rhor = G.rhor[irnew];
                    }
                    if (p.E <= T.ecut) ecut_discard = true;
                    else if (s.medium != medold) { s.state = 1; continue; }
                    else {
                        // $UPDATE-DEMFP (src/egsnrc.macros:3273-3281)
                        s.demfp = s.demfp - (Real)(de * (Real)sig);
                        s.total_de = s.total_de - de;
                        s.total_tstep = s.total_tstep - (Real)tvstep * (Real)rhof;
                        if (s.total_tstep < (Real)1e-9) s.demfp = 0;
                        if (!(s.demfp < (Real)1e-8)) continue;
                        // fictitious-cross-section rejection
                        const MedScalars<Real> &M2 = cmed<Real>(s.medium);
                        ERow<Real> ef{erow(T, M2, s.lelke), qel};
                        Real sigf = ef.sig(s.elke) / ef.dedx(s.elke);
                        Real rfict = urand<Real>(p.rng);
                        if (!(rfict <= sigf / s.sig0)) { s.state = 1; continue; }
                        s.state = 3;   // interaction due: wait for the warp's batch
                        continue;
                    }
                }
            }
        }
        // :ECUT-DISCARD: (src/egsnrc.mortran:1768-1802)
        {
            Real edep = p.E - rm;
            deposit(P, acc, p.ir, p.rng.hist, edep * p.wt);
            edep_tot += (double)(edep * p.wt);
            if (Adj) elist_flush(P, el);
            if (p.iq > 0) annih_at_rest(P, P.pout, p, npush, err);
            alive = false;
        }
    }
    acc_flush(P, acc);
    edep_tot += (double)edep_part;
    for (int o = 16; o > 0; o >>= 1) {
        nstep += __shfl_down_sync(0xffffffffu, nstep, o);
        npush += __shfl_down_sync(0xffffffffu, npush, o);
        ninter += __shfl_down_sync(0xffffffffu, ninter, o);
        edep_tot += __shfl_down_sync(0xffffffffu, edep_tot, o);
        esc_tot += __shfl_down_sync(0xffffffffu, esc_tot, o);
        if (SPLIT) nwide += __shfl_down_sync(0xffffffffu, nwide, o);
    }
    if (lane == 0) {
        if (SPLIT) atomicAdd(P.counters + CNT_EWIDE, nwide);
        atomicAdd(P.counters + CNT_ELANES, lanes);
        atomicAdd(P.counters + CNT_EITER, iters);
        atomicAdd(P.counters + CNT_ESTEP, nstep);
        atomicAdd(P.counters + CNT_EPUSH, npush);
        atomicAdd(P.counters + CNT_EINTER, ninter);
        atomicAdd(P.energy + 0, edep_tot);
        atomicAdd(P.energy + 1, esc_tot);
    }
    if (err) atomicExch(P.error + 1, 1);
}

// Batch fold: sum += d, sum2 += d*d, d = 0 (DOSXYZnrc batch statistics).
__global__ void k_batch(double *d, double *sum, double *sum2, long long n) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    long long stride = (long long)gridDim.x * blockDim.x;
    for (; i < n; i += stride) {
        double x = d[i];
        sum[i] += x;
        sum2[i] += x * x;
        d[i] = 0;
    }
}

// Loop control of the device-side wavefront loop (egsgpu_config.use_graph = 2):
// runs after each pair of rounds inside a conditional WHILE graph node and
// keeps the loop going while either next input queue (photon queue 0, count
// counts[0]; electron queue 2, count counts[4]) holds particles, for at most
// `limit` rounds; a loop stopped by the limit sets the loop-cap error flag.
__global__ void k_rounds(cudaGraphConditionalHandle hc, const unsigned *counts, unsigned *rounds, unsigned limit,
                         int *error) {
    const unsigned r = (rounds[0] += 2);
    bool more = counts[0] != 0 || counts[4] != 0;
    if (more && r >= limit) {
        error[1] = 1;
        more = false;
    }
    cudaGraphSetConditional(hc, more ? 1u : 0u);
}

// Geometry queries on one phantom through the transport kernels' own
// functions (a checking aid): op 0 isWhere of x; op 1 howfar from region
// ireg (howfarFromOut when ireg < 0) along u within t, writing the new region
// and the distance; op 2 hownear of x in region ireg.  The host checks every
// region index against the phantom before the launch.
template <class Real>
__global__ void k_geometry_query(Geom<Real> G, int op, long long n, const int *ireg, const double *x, const double *u,
                                 double *t, int *inew) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double *p = x + 3 * i;
    if (op == 0) {
        int ix = plane_where(G.xb, G.nx, (Real)p[0]), iy = plane_where(G.yb, G.ny, (Real)p[1]);
        int iz = plane_where(G.zb, G.nz, (Real)p[2]);
        inew[i] = (ix >= 0 && iy >= 0 && iz >= 0) ? G.voff + ix + iy * G.nx + iz * G.nxy : -1;
    } else if (op == 1) {
        const double *d = u + 3 * i;
        if (ireg[i] >= 0) {
            Real tt = (Real)t[i];
            inew[i] = howfar(G, ireg[i], (Real)p[0], (Real)p[1], (Real)p[2], (Real)d[0], (Real)d[1], (Real)d[2], tt);
            t[i] = (double)tt;
        } else {
            double tt = t[i];
            inew[i] = howfar_from_out(G, p, d, tt);
            t[i] = tt;
        }
    } else {
        t[i] = (double)hownear(G, ireg[i], (Real)p[0], (Real)p[1], (Real)p[2]);
    }
}

}  // namespace EGSGPU_TU
}  // namespace egsgpu

// ===================================================================
//                         host-side engine
// ===================================================================
using namespace egsgpu;
using namespace egsgpu::EGSGPU_TU;

namespace egsgpu_host {

#define CK(x)                                                                                 \
    do {                                                                                      \
        cudaError_t e_ = (x);                                                                 \
        if (e_ != cudaSuccess) {                                                              \
            err = std::string(#x) + ": " + cudaGetErrorString(e_);                            \
            return EGSGPU_ERR_CUDA;                                                           \
        }                                                                                     \
    } while (0)

// One phantom of a multi-phantom run, as handed to the engine.
struct PhantomDesc {
    int nx, ny, nz;
    const double *xb, *yb, *zb;
    const int32_t *med;
    const double *rhor;
    uint32_t seed;
    long long histories;
};

// The engine behind a handle: one implementation per precision (Engine<float>
// here, Engine<double> in the FP64 translation unit).
struct EngineBase {
    virtual ~EngineBase() {}
    virtual int load(const egs::Hatch &H, double ecut, double pcut, double skindepth, double smax,
                     std::string &err) = 0;
    virtual int geometry(int nx, int ny, int nz, const double *xb, const double *yb, const double *zb,
                         const int32_t *med, const double *rhor, std::string &err) = 0;
    virtual int run(const Source &S, long long first, long long n, int nbatch, uint32_t seed, cudaStream_t st,
                    std::string &err) = 0;
    virtual int run_noalloc(const Source &S, long long first, long long n, uint32_t seed, double *dose,
                            cudaStream_t st, unsigned char *scratch, size_t scratch_bytes, std::string &err) = 0;
    virtual int problems(int n, const PhantomDesc *pd, const Source *src, std::string &err) = 0;
    virtual int run_multi(const Source &Smax, int nbatch, cudaStream_t st, std::string &err) = 0;
    virtual int adjoint(const Source &S, long long first, long long n, uint32_t seed, const double *w, double *grad,
                        std::string &err) = 0;
    // tallies and counters of the runs so far
    virtual int clear_tallies(long long nv, std::string &err) = 0;
    virtual int read_sums(long long off, long long n, double *sum, double *sum2, std::string &err) = 0;
    virtual int read_totals(double *energy2, unsigned long long *counters, std::string &err) = 0;   // CNT_N counters
    virtual int restore_sums(const double *energy2, const unsigned long long *counters8, const double *sum,
                             const double *sum2, long long nv, std::string &err) = 0;
    virtual int read_profile(double *out20, std::string &err) = 0;
    virtual int history_tally(long long first, long long n, std::string &err) = 0;
    virtual int read_history_tally(double *out, std::string &err) = 0;
    virtual int geometry_query(int op, long long n, const int *ireg, const double *x, const double *u, double *t,
                               int *inew, std::string &err) = 0;
};

// The FP64 engine, built in its own translation unit (egs_transport_f64.cu).
EngineBase *make_engine_f64(const egsgpu_config &c);

namespace EGSGPU_TU {

// Multiplier and shift for dividing by d with a multiply-high, an add and a
// shift: l = ceil(log2 d), m = floor(2^32 (2^l - d) / d) + 1; then
// n / d = (umulhi(n, m) + n) >> l for 0 <= n < 2^31 (the sum cannot overflow).
static void fast_divisor(uint32_t d, uint32_t &m, int &l) {
    l = 0;
    while ((1ull << l) < d) ++l;
    m = (uint32_t)((((1ull << 32) * ((1ull << l) - d)) / d) + 1);
}
// Runs f(begin, end) over the index range [0, n), split over up to 16 host
// threads; small ranges run on the calling thread.  Used for the per-voxel
// host loops of the phantom uploads (tens of millions of voxels per step for
// a caller that uploads its phantoms every time).
template <class F>
static void host_parallel(long long n, F f) {
    unsigned t = std::min(16u, std::max(1u, std::thread::hardware_concurrency()));
    if (n < (1LL << 20) || t == 1) { f(0LL, n); return; }
    std::vector<std::thread> th;
    const long long per = (n + t - 1) / t;
    for (unsigned k = 0; k < t; ++k) {
        const long long b = k * per, e = std::min(n, b + per);
        if (b < e) th.emplace_back(f, b, e);
    }
    for (auto &x : th) x.join();
}

// Calls f(k, begin, end) for the voxels [begin, end) of phantom k, over n
// phantoms laid end to end (phantom k's voxels are [off[k], off[k+1]) of the
// global range), split over host threads by the global range.
template <class F>
static void phantoms_parallel(const std::vector<long long> &off, F f) {
    const int n = (int)off.size() - 1;
    host_parallel(off[n], [&](long long b, long long e) {
        int k = (int)(std::upper_bound(off.begin(), off.end(), b) - off.begin()) - 1;
        for (long long i = b; i < e;) {
            while (i >= off[k + 1]) ++k;
            const long long stop = std::min(e, off[k + 1]);
            f(k, i - off[k], stop - off[k]);
            i = stop;
        }
    });
}

// An allocator whose resize() leaves new elements of trivial types
// uninitialised: the voxel copies overwrite every element, and zero-filling
// a gigabyte first costs more than the copy itself.
template <class T>
struct NoInitAlloc : std::allocator<T> {
    template <class U> struct rebind { using other = NoInitAlloc<U>; };
    NoInitAlloc() = default;
    template <class U> NoInitAlloc(const NoInitAlloc<U> &) noexcept {}
    template <class U> void construct(U *p) noexcept { ::new ((void *)p) U; }
    template <class U, class... A> void construct(U *p, A &&...a) { ::new ((void *)p) U(std::forward<A>(a)...); }
};
template <class T>
using raw_vector = std::vector<T, NoInitAlloc<T>>;

// Checks the medium indices and relative densities of nv voxels: 0, or 1 for
// a medium index out of range, 2 for a density that is not positive and finite.
static int check_range(long long nv, const int32_t *med, const double *rhor, int nmed) {
    for (long long i = 0; i < nv; ++i) {
        if (med[i] < 0 || med[i] >= nmed) return 1;
        if (!(rhor[i] > 0) || !std::isfinite(rhor[i])) return 2;
    }
    return 0;
}
// The same over host threads.
static int check_voxels(long long nv, const int32_t *med, const double *rhor, int nmed) {
    std::atomic<int> bad{0};
    host_parallel(nv, [&](long long b, long long e) {
        if (int v = check_range(e - b, med + b, rhor + b, nmed)) bad.fetch_or(v);
    });
    const int v = bad.load();
    return (v & 1) ? 1 : (v & 2) ? 2 : 0;
}

template <class Real>
static void set_divisors(Geom<Real> &g) {
    fast_divisor((uint32_t)g.nx, g.mnx, g.lnx);
    fast_divisor((uint32_t)g.nxy, g.mnxy, g.lnxy);
}

struct DevMem {
    void *p = nullptr;
    size_t n = 0;   // bytes allocated
    ~DevMem() { if (p) cudaFree(p); }
    // Keeps the current allocation when it is large enough, so that a caller
    // who uploads a phantom of the same size every step allocates nothing
    // (cudaMalloc and cudaFree synchronise the device).
    cudaError_t alloc(size_t bytes) {
        const size_t want = bytes ? bytes : 16;
        if (p && want <= n) return cudaSuccess;
        if (p) { cudaFree(p); p = nullptr; n = 0; }
        cudaError_t e = cudaMalloc(&p, want);
        if (e == cudaSuccess) n = want;
        else p = nullptr;
        return e;
    }
};

template <class Real>
struct Engine : EngineBase {
    egsgpu_config cfg;

    int clear_tallies(long long nv, std::string &err) override {
        CK(cudaMemset(d_dose.p, 0, nv * sizeof(double)));
        CK(cudaMemset(d_sum.p, 0, nv * sizeof(double)));
        CK(cudaMemset(d_sum2.p, 0, nv * sizeof(double)));
        CK(cudaMemset(d_energy.p, 0, 2 * sizeof(double)));
        CK(cudaMemset(d_counters.p, 0, CNT_N * sizeof(unsigned long long)));
        CK(cudaMemset(d_error.p, 0, 2 * sizeof(int)));
        for (int k = 0; k < 4; ++k) { prof_ms[k] = 0; prof_n[k] = 0; }
        return 0;
    }
    int read_sums(long long off, long long n, double *sum, double *sum2, std::string &err) override {
        if (sum) CK(cudaMemcpy(sum, (double *)d_sum.p + off, n * sizeof(double), cudaMemcpyDeviceToHost));
        if (sum2) CK(cudaMemcpy(sum2, (double *)d_sum2.p + off, n * sizeof(double), cudaMemcpyDeviceToHost));
        return 0;
    }
    int read_totals(double *energy2, unsigned long long *counters, std::string &err) override {
        if (energy2) CK(cudaMemcpy(energy2, d_energy.p, 2 * sizeof(double), cudaMemcpyDeviceToHost));
        if (counters) CK(cudaMemcpy(counters, d_counters.p, CNT_N * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
        return 0;
    }
    int restore_sums(const double *energy2, const unsigned long long *counters8, const double *sum,
                     const double *sum2, long long nv, std::string &err) override {
        CK(cudaMemcpy(d_energy.p, energy2, 2 * sizeof(double), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(d_counters.p, counters8, 8 * sizeof(unsigned long long), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(d_sum.p, sum, nv * sizeof(double), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(d_sum2.p, sum2, nv * sizeof(double), cudaMemcpyHostToDevice));
        CK(cudaMemset(d_dose.p, 0, nv * sizeof(double)));
        return 0;
    }
    int read_profile(double *out, std::string &err) override {
        unsigned long long c[CNT_N];
        CK(cudaMemcpy(c, d_counters.p, sizeof(c), cudaMemcpyDeviceToHost));
        for (int k = 0; k < 4; ++k) { out[k] = prof_ms[k]; out[4 + k] = (double)prof_n[k]; }
        out[8] = (double)c[CNT_PSTEP]; out[9] = (double)c[CNT_ESTEP];
        out[10] = (double)c[CNT_PUSH]; out[11] = (double)c[CNT_EPUSH];
        out[12] = (double)c[CNT_INTER]; out[13] = (double)c[CNT_EINTER];
        out[14] = (double)tuned_chunk;
        out[15] = gexec_loop ? 2.0 : (gexec ? 1.0 : 0.0);
        out[16] = c[CNT_PITER] ? (double)c[CNT_PLANES] / c[CNT_PITER] : 0.0;
        out[17] = c[CNT_EITER] ? (double)c[CNT_ELANES] / c[CNT_EITER] : 0.0;
        out[18] = (double)c[CNT_EWIDE];
        out[19] = (double)shape_sel;
        return 0;
    }
    int history_tally(long long first, long long n, std::string &err) override {
        hist_first = first;
        hist_n = n;
        if (n > 0) {
            CK(d_hist.alloc(n * sizeof(double)));
            CK(cudaMemset(d_hist.p, 0, n * sizeof(double)));
        }
        return 0;
    }
    int read_history_tally(double *out, std::string &err) override {
        if (hist_n > 0) CK(cudaMemcpy(out, d_hist.p, hist_n * sizeof(double), cudaMemcpyDeviceToHost));
        return 0;
    }

    int geometry_query(int op, long long n, const int *ireg, const double *x, const double *u, double *t, int *inew,
                       std::string &err) override {
        if (!G.xb || nprob) { err = "a single geometry must be set"; return EGSGPU_ERR_STATE; }
        if (op < 0 || op > 2 || n < 0 || !x || (op != 0 && (!ireg || !t)) || (op == 1 && !u) || (op != 2 && !inew)) {
            err = "geometry query: bad arguments";
            return EGSGPU_ERR_ARG;
        }
        if (n == 0) return 0;
        if (op != 0)
            for (long long i = 0; i < n; ++i)
                if (ireg[i] >= nvox || (op == 2 && ireg[i] < 0)) { err = "geometry query: region out of range"; return EGSGPU_ERR_ARG; }
        DevMem dreg, dx, du, dt, dnew;
        CK(dreg.alloc(n * sizeof(int)));
        CK(dx.alloc(3 * n * sizeof(double)));
        CK(du.alloc(3 * n * sizeof(double)));
        CK(dt.alloc(n * sizeof(double)));
        CK(dnew.alloc(n * sizeof(int)));
        CK(cudaMemcpy(dx.p, x, 3 * n * sizeof(double), cudaMemcpyHostToDevice));
        if (op != 0) CK(cudaMemcpy(dreg.p, ireg, n * sizeof(int), cudaMemcpyHostToDevice));
        if (op == 1) CK(cudaMemcpy(du.p, u, 3 * n * sizeof(double), cudaMemcpyHostToDevice));
        if (op == 1) CK(cudaMemcpy(dt.p, t, n * sizeof(double), cudaMemcpyHostToDevice));
        k_geometry_query<Real><<<(unsigned)((n + 255) / 256), 256>>>(G, op, n, (const int *)dreg.p, (const double *)dx.p,
                                                                     (const double *)du.p, (double *)dt.p, (int *)dnew.p);
        CK(cudaGetLastError());
        CK(cudaDeviceSynchronize());
        if (op != 0) CK(cudaMemcpy(t, dt.p, n * sizeof(double), cudaMemcpyDeviceToHost));
        if (op != 2) CK(cudaMemcpy(inew, dnew.p, n * sizeof(int), cudaMemcpyDeviceToHost));
        return 0;
    }

    int nmed = 0;
    std::vector<MedScalars<Real>> meds;
    DevMem d_etab, d_erange, d_gtab, d_pmax, d_ray, d_rayi, d_shell, d_shellat, d_elem, d_ms, d_msi;
    Tables<Real> T{};
    // geometry
    Geom<Real> G{};
    DevMem d_xb, d_yb, d_zb, d_med, d_rhor;
    long long nvox = 0;
    // queues: P[2], E[2]
    DevMem qmem[4];
    Queue<Real> q[4];
    DevMem d_counts;   // 4 queues x (count, head)
    unsigned capacity = 0;
    // tallies
    DevMem d_dose, d_sum, d_sum2, d_energy, d_counters, d_error, d_hist;
    long long hist_first = 0, hist_n = 0;
    int sm_count = 0;
    // per-kernel device time (CUDA events on the launch stream) and launches:
    // 0 source, 1 photon, 2 electron, 3 batch
    double prof_ms[4] = {0, 0, 0, 0};
    long long prof_n[4] = {0, 0, 0, 0};
    cudaEvent_t ev[8] = {};
    bool events_ready = false;
    // Launch-shape candidates: threads per CTA, and resident CTAs per SM of the
    // photon and electron kernels relative to the most that fit.
    struct Shape { int bs, dp, de; };
    static constexpr int NSHAPES = 6;
    static constexpr Shape SHAPES[NSHAPES] = {{128, 0, 0}, {64, 0, 0}, {96, 0, 0}, {128, 0, -1}, {128, -2, 0},
                                              {64, 0, -2}};
    int shape_try = 0, shape_sel = -1;   // next candidate to time; chosen candidate (-1: not yet)
    long long shape_cn = 0;              // histories of the chunks the candidates are timed on
    double shape_rate[NSHAPES] = {};
    long long tuned_chunk = 0;   // histories per wavefront chosen by the autotuner
    long long best_chunk = 0;
    double best_rate = 0;
    bool tune_done = false;

    explicit Engine(const egsgpu_config &c) : cfg(c) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, dev);
    }
    ~Engine() {
        if (gexec) cudaGraphExecDestroy(gexec);
        if (gexec_loop) cudaGraphExecDestroy(gexec_loop);
        if (events_ready) {
            for (auto &e : ev) cudaEventDestroy(e);
            for (auto &e : gev) cudaEventDestroy(e);
            cudaEventDestroy(ev_in);
            cudaStreamDestroy(ws);
        }
    }
    // accumulate the elapsed time between events 2k and 2k+1 (after a sync)
    void prof_take(int k, int slot) {
        float ms = 0;
        if (cudaEventElapsedTime(&ms, ev[2 * slot], ev[2 * slot + 1]) == cudaSuccess) {
            prof_ms[k] += ms;
            ++prof_n[k];
        }
    }

    int load(const egs::Hatch &H, double ecut, double pcut, double skindepth, double smax,
             std::string &err) override {
        nmed = (int)H.media.size();
        if (nmed > MAXMED) { err = "too many media"; return EGSGPU_ERR_ARG; }
        std::vector<Real> etab, gtab, pmax, ray, shell, elem, ms;
        std::vector<Real> erange;
        std::vector<int> rayi, shellat, msi;
        meds.assign(nmed, MedScalars<Real>());
        int eoff = 0, goff = 0, soff = 0, loff = 0;
        for (int im = 0; im < nmed; ++im) {
            const egs::Medium &m = H.media[im];
            MedScalars<Real> &M = meds[im];
            std::memset(&M, 0, sizeof(M));
            M.rho = (Real)m.rho; M.ae = (Real)m.ae; M.ap = (Real)m.ap; M.te = (Real)m.te;
            M.thmoll = (Real)m.thmoll; M.blcc = (Real)m.blcc; M.xcc = (Real)m.xcc;
            M.eke0 = (Real)m.eke0; M.eke1 = (Real)m.eke1; M.ge0 = (Real)m.ge0; M.ge1 = (Real)m.ge1;
            M.esig_e = (Real)m.esig_e; M.psig_e = (Real)m.psig_e; M.log_ap = (Real)m.log_ap;
            M.delcm = (Real)m.delcm; M.zbrang = (Real)m.zbrang; M.lzbrang = (Real)m.lzbrang;
            for (int k = 0; k < 6; ++k)
                for (int l = 0; l < 8; ++l) M.dl[k][l] = (Real)m.dl[k][l];
            M.bpar[0] = (Real)m.bpar[0]; M.bpar[1] = (Real)m.bpar[1];
            M.E_array0 = (Real)m.E_array[0];
            M.meke = m.meke; M.n_shell = m.n_shell; M.nne = m.nne;
            M.sig_mono_e = m.sig_ismonotone[0]; M.sig_mono_p = m.sig_ismonotone[1];
            M.etab_off = eoff; M.gtab_off = goff; M.shell_off = soff; M.elem_off = loff;
            if (m.nne > MAXNE) { err = "too many elements in medium " + m.name; return EGSGPU_ERR_ARG; }
            for (int k = 0; k < m.nne; ++k) M.pz[k] = (float)m.pz[k];
            for (int i = 0; i < m.meke; ++i) {
                const double v[16] = {m.esig0[i], m.esig1[i], m.psig0[i], m.psig1[i], m.ededx0[i], m.ededx1[i],
                                      m.pdedx0[i], m.pdedx1[i], m.ebr10[i], m.ebr11[i], m.pbr10[i], m.pbr11[i],
                                      m.pbr20[i], m.pbr21[i], m.tmxs0[i], m.tmxs1[i]};
                for (double x : v) etab.push_back((Real)x);
                erange.push_back((Real)m.E_array[i]); erange.push_back((Real)m.range_ep0[i]);
                erange.push_back((Real)m.range_ep1[i]); erange.push_back(0);
            }
            eoff += m.meke;
            for (int i = 0; i < m.mge; ++i) {
                const double v[8] = {m.gmfp0[i], m.gmfp1[i], m.gbr10[i], m.gbr11[i],
                                     m.gbr20[i], m.gbr21[i], m.cohe0[i], m.cohe1[i]};
                for (double x : v) gtab.push_back((Real)x);
                pmax.push_back((Real)m.pmax0[i]); pmax.push_back((Real)m.pmax1[i]);
            }
            if (m.mge != MXGE) { err = "unexpected photon grid size"; return EGSGPU_ERR_DATA; }
            goff += m.mge;
            for (int i = 0; i < NRAY; ++i) ray.push_back((Real)m.xgrid[i]);
            for (int i = 0; i < NRAY; ++i) ray.push_back((Real)m.fcum[i]);
            for (int i = 0; i < NRAY; ++i) ray.push_back((Real)m.b_array[i]);
            for (int i = 0; i < NRAY; ++i) ray.push_back((Real)m.c_array[i]);
            for (int i = 0; i < NRAY; ++i) rayi.push_back(m.i_array[i]);
            for (int i = 0; i < m.n_shell; ++i) {
                int j = m.shell_array[i];
                shell.push_back((Real)m.eno_array[i]); shell.push_back((Real)H.shells.be[j]);
                shell.push_back((Real)H.shells.Jo[j]); shell.push_back((Real)H.shells.erfJo[j]);
                shellat.push_back(m.eno_atbin_array[i]);
            }
            soff += m.n_shell;
            for (int k = 0; k < m.nne; ++k) {
                const egs::ElementPhoto &e = H.elements[m.elem_index[k]];
                Real row[96] = {};
                for (int j = 0; j < 16; ++j) {
                    row[j] = (Real)e.edge_a[j]; row[16 + j] = (Real)e.edge_b[j]; row[32 + j] = (Real)e.edge_c[j];
                    row[48 + j] = (Real)e.edge_d[j]; row[64 + j] = (Real)e.edge_energies[j];
                }
                for (int j = 0; j < 6; ++j) { row[80 + j] = (Real)e.binding[j]; row[86 + j] = (Real)e.interaction_prob[j]; }
                row[95] = (Real)e.edge_number;
                elem.insert(elem.end(), row, row + 96);
            }
            loff += m.nne;
        }
        for (size_t i = 0; i < H.ums.size(); ++i) {
            ms.push_back((Real)H.ums[i]); ms.push_back((Real)H.fms[i]); ms.push_back((Real)H.wms[i]);
            msi.push_back(H.ims[i]);
        }
        auto up = [&](DevMem &d, const void *src, size_t bytes) -> cudaError_t {
            cudaError_t e = d.alloc(bytes);
            if (e != cudaSuccess) return e;
            return cudaMemcpy(d.p, src, bytes, cudaMemcpyHostToDevice);
        };
        CK(up(d_etab, etab.data(), etab.size() * sizeof(Real)));
        h_etab = etab;
        hatch_ = &H;
        CK(up(d_erange, erange.data(), erange.size() * sizeof(Real)));
        CK(up(d_gtab, gtab.data(), gtab.size() * sizeof(Real)));
        CK(up(d_pmax, pmax.data(), pmax.size() * sizeof(Real)));
        CK(up(d_ray, ray.data(), ray.size() * sizeof(Real)));
        CK(up(d_rayi, rayi.data(), rayi.size() * sizeof(int)));
        CK(up(d_shell, shell.data(), shell.size() * sizeof(Real)));
        CK(up(d_shellat, shellat.data(), shellat.size() * sizeof(int)));
        CK(up(d_elem, elem.data(), elem.size() * sizeof(Real)));
        CK(up(d_ms, ms.data(), ms.size() * sizeof(Real)));
        CK(up(d_msi, msi.data(), msi.size() * sizeof(int)));
        if (sizeof(Real) == 4) CK(cudaMemcpyToSymbol(c_med_f, meds.data(), nmed * sizeof(MedScalars<Real>)));
        else CK(cudaMemcpyToSymbol(c_med_d, meds.data(), nmed * sizeof(MedScalars<Real>)));
        T.etab = (const Real *)d_etab.p; T.erange = (const Real *)d_erange.p; T.gtab = (const Real *)d_gtab.p;
        T.pmax = (const Real *)d_pmax.p; T.ray = (const Real *)d_ray.p; T.ray_i = (const int *)d_rayi.p;
        T.shell = (const Real *)d_shell.p; T.shell_at = (const int *)d_shellat.p; T.elem = (const Real *)d_elem.p;
        T.ms = (const Real *)d_ms.p; T.ms_i = (const int *)d_msi.p;
        T.dllambi = (Real)H.dllambi; T.dqmsi = (Real)H.dqmsi;
        T.nmed = nmed;
        T.ecut = (Real)ecut; T.pcut = (Real)pcut; T.skindepth = (Real)skindepth; T.smaxir = (Real)smax;
        // tallies that do not depend on the geometry
        CK(d_energy.alloc(2 * sizeof(double)));
        CK(d_counters.alloc(CNT_N * sizeof(unsigned long long)));
        CK(d_error.alloc(2 * sizeof(int)));
        CK(cudaMemset(d_energy.p, 0, 2 * sizeof(double)));
        CK(cudaMemset(d_counters.p, 0, CNT_N * sizeof(unsigned long long)));
        CK(cudaMemset(d_error.p, 0, 2 * sizeof(int)));
        return 0;
    }

    // HOWFARLESS: the phantom must be one medium at one density; the step
    // limits use the smallest voxel dimension (egs_hatch.cpp howfarless_tmxs)
    bool homogeneous = false;
    double mindel = 0, hfl_mindel = -1;
    const egs::Hatch *hatch_ = nullptr;
    std::vector<Real> h_etab;
    DevMem d_etab_hfl;

    int hfl_tables(std::string &err) {
        if (hfl_mindel == mindel && d_etab_hfl.p) return 0;
        std::vector<Real> e = h_etab;
        for (int im = 0; im < nmed; ++im) {
            std::vector<double> t0, t1;
            egs::howfarless_tmxs(hatch_->media[im], hatch_->params, mindel, t0, t1);
            for (int i = 0; i < hatch_->media[im].meke; ++i) {
                e[((size_t)meds[im].etab_off + i) * 16 + 14] = (Real)t0[i];
                e[((size_t)meds[im].etab_off + i) * 16 + 15] = (Real)t1[i];
            }
        }
        CK(d_etab_hfl.alloc(e.size() * sizeof(Real)));
        CK(cudaMemcpy(d_etab_hfl.p, e.data(), e.size() * sizeof(Real), cudaMemcpyHostToDevice));
        hfl_mindel = mindel;
        return 0;
    }

    int geometry(int nx, int ny, int nz, const double *xb, const double *yb, const double *zb, const int32_t *med,
                 const double *rhor, std::string &err) override {
        nprob = 0;
        nvox = (long long)nx * ny * nz;
        std::atomic<bool> mixed{false};
        host_parallel(nvox, [&](long long b, long long e) {
            for (long long i = b; i < e && !mixed.load(std::memory_order_relaxed); ++i)
                if (med[i] != med[0] || rhor[i] != rhor[0]) mixed.store(true);
        });
        homogeneous = !mixed.load();
        mindel = 1e30;
        for (int i = 0; i < nx; ++i) mindel = std::min(mindel, xb[i + 1] - xb[i]);
        for (int i = 0; i < ny; ++i) mindel = std::min(mindel, yb[i + 1] - yb[i]);
        for (int i = 0; i < nz; ++i) mindel = std::min(mindel, zb[i + 1] - zb[i]);
        std::vector<Real> x(xb, xb + nx + 1), y(yb, yb + ny + 1), z(zb, zb + nz + 1);
        raw_vector<Real> r(nvox);
        raw_vector<uint8_t> m(nvox);
        host_parallel(nvox, [&](long long b, long long e) {
            for (long long i = b; i < e; ++i) { m[i] = (uint8_t)med[i]; r[i] = (Real)rhor[i]; }
        });
        auto up = [&](DevMem &d, const void *src, size_t bytes) -> cudaError_t {
            cudaError_t e = d.alloc(bytes);
            if (e != cudaSuccess) return e;
            return cudaMemcpy(d.p, src, bytes, cudaMemcpyHostToDevice);
        };
        CK(up(d_xb, x.data(), x.size() * sizeof(Real)));
        CK(up(d_yb, y.data(), y.size() * sizeof(Real)));
        CK(up(d_zb, z.data(), z.size() * sizeof(Real)));
        CK(up(d_med, m.data(), m.size()));
        CK(up(d_rhor, r.data(), r.size() * sizeof(Real)));
        G.nx = nx; G.ny = ny; G.nz = nz; G.nxy = nx * ny;
        G.xb = (const Real *)d_xb.p; G.yb = (const Real *)d_yb.p; G.zb = (const Real *)d_zb.p;
        G.med = (const uint8_t *)d_med.p; G.rhor = (const Real *)d_rhor.p;
        // egs++ distanceEpsilon: 2^-32 cm in FP64, 2^-21 cm in FP32 (egs++/egs_functions.h:80-88)
        G.bt = sizeof(Real) == 8 ? (Real)(1.0 / 4294967296.0) : (Real)(1.0 / 2097152.0);
        G.hbt = G.bt / 2;
        G.voff = 0;
        set_divisors(G);
        CK(d_dose.alloc(nvox * sizeof(double)));
        CK(d_sum.alloc(nvox * sizeof(double)));
        CK(d_sum2.alloc(nvox * sizeof(double)));
        CK(cudaMemset(d_dose.p, 0, nvox * sizeof(double)));
        CK(cudaMemset(d_sum.p, 0, nvox * sizeof(double)));
        CK(cudaMemset(d_sum2.p, 0, nvox * sizeof(double)));
        return 0;
    }

    static constexpr size_t QUEUE_RECORD = 12 * sizeof(Real) + sizeof(int) + 2 * sizeof(int8_t) +
                                           2 * sizeof(uint32_t) + sizeof(unsigned long long);
    // Records per queue when egsgpu_config.capacity is 0: the largest power of
    // two from 2^27 down to 2^20 whose four queues take at most a sixth of the
    // device memory free when the handle first runs (2^27 on a GB300 with
    // nothing else resident: 37.6 GB in FP32).  Larger queues let the chunk
    // autotuner run more histories per wavefront, and each chunk ends in a few
    // short, sparsely occupied rounds: a 64^3-voxel slab phantom under a
    // 0.1-6 MeV photon field runs 6% faster at 2^27 than at 2^25.  Results do
    // not depend on the capacity.
    unsigned default_capacity() {
        if (capacity > 0) return capacity;
        size_t fr = 0, tot = 0;
        if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) { cudaGetLastError(); return 1u << 25; }
        for (int b = 27; b > 20; --b)
            if (4 * (((size_t)1 << b) * QUEUE_RECORD + 1024) <= fr / 6) return 1u << b;
        return 1u << 20;
    }
    int ensure_queues(unsigned cap, std::string &err) {
        if (cap <= capacity) return 0;
        const size_t per = QUEUE_RECORD;
        CK(d_counts.alloc(16 * sizeof(unsigned)));
        for (int k = 0; k < 4; ++k) {
            CK(qmem[k].alloc((size_t)cap * per + 1024));
            char *b = (char *)qmem[k].p;
            auto take = [&](size_t bytes) { char *r = b; b += (bytes + 255) & ~(size_t)255; return r; };
            Queue<Real> &Q = q[k];
            Q.x = (Real *)take(cap * sizeof(Real)); Q.y = (Real *)take(cap * sizeof(Real));
            Q.z = (Real *)take(cap * sizeof(Real)); Q.u = (Real *)take(cap * sizeof(Real));
            Q.v = (Real *)take(cap * sizeof(Real)); Q.w = (Real *)take(cap * sizeof(Real));
            Q.E = (Real *)take(cap * sizeof(Real)); Q.wt = (Real *)take(cap * sizeof(Real));
            Q.ir = (int *)take(cap * sizeof(int));
            Q.iq = (k >= 2) ? (int8_t *)take(cap) : nullptr;
            Q.hist = (uint32_t *)take(cap * sizeof(uint32_t)); Q.n = (uint32_t *)take(cap * sizeof(uint32_t));
            Q.sid = (unsigned long long *)take(cap * sizeof(unsigned long long));
            Q.st = (uint8_t *)take(cap);
            Q.aux0 = (Real *)take(cap * sizeof(Real));
            Q.aux1 = (k >= 2) ? (Real *)take(cap * sizeof(Real)) : nullptr;
            Q.aux2 = (k >= 2) ? (Real *)take(cap * sizeof(Real)) : nullptr;
            Q.aux3 = (k >= 2) ? (Real *)take(cap * sizeof(Real)) : nullptr;
            Q.count = (unsigned *)d_counts.p + 2 * k;
            Q.capacity = cap;
        }
        capacity = cap;
        return 0;
    }

    // ROUNDS wavefront rounds (photon kernel, then electron kernel, on
    // alternating queue pairs; a launch whose queue is empty retires at once)
    // are enqueued back to back and the host reads the queue counters once
    // per ROUNDS, so host-side stalls do not idle the GPU between rounds.  The
    // rounds are either launched directly, with CUDA events around every
    // kernel, or replayed from a CUDA graph of the same launches.
    static constexpr int ROUNDS = 4;
    cudaStream_t ws = nullptr;
    cudaGraphExec_t gexec = nullptr;
    cudaEvent_t gev[4 * ROUNDS] = {};
    cudaEvent_t ev_in = nullptr;
    bool graph_ok = true;

    // The EXACT electron kernel, or its precision-split instantiation in the
    // FP32 engine when egsgpu_config.fp64_near_faces is set (PRESTA-I,
    // HOWFARLESS and the adjoint keep their own kernels).
    template <bool M>
    void launch_electron(const Params<Real> &P, int ge, int bs) {
        if constexpr (sizeof(Real) == 4) {
            if (cfg.fp64_near_faces > 0) {
                k_electron<Real, M, false, false, false, true><<<ge, bs, 0, ws>>>(P);
                return;
            }
        }
        k_electron<Real, M><<<ge, bs, 0, ws>>>(P);
    }
    template <bool M>
    cudaError_t electron_occupancy(int &occ, int bs) {
        if constexpr (sizeof(Real) == 4) {
            if (cfg.fp64_near_faces > 0)
                return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_electron<Real, M, false, false, false, true>, bs, 0);
        }
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_electron<Real, M>, bs, 0);
    }

    cudaError_t enqueue_rounds(const Params<Real> &P0, int gp, int ge, int bs, bool events, bool multi,
                               bool adj = false, bool hfl = false, int nrounds = ROUNDS) {
        const bool pi = cfg.bca_algorithm == 1;
        unsigned *counts = (unsigned *)d_counts.p;
        cudaError_t e = cudaSuccess;
        for (int r = 0; r < nrounds && e == cudaSuccess; ++r) {
            int cur = r & 1, nxt = 1 - cur;
            Params<Real> P = P0;
            P.pin = q[cur]; P.ein = q[2 + cur]; P.pout = q[nxt]; P.eout = q[2 + nxt];
            if ((e = cudaMemsetAsync(counts + 2 * nxt, 0, 2 * sizeof(unsigned), ws))) break;
            if ((e = cudaMemsetAsync(counts + 4 + 2 * nxt, 0, 2 * sizeof(unsigned), ws))) break;
            if (events && (e = cudaEventRecord(gev[4 * r], ws))) break;
            if (hfl) k_photon<Real, false, false, true><<<gp, bs, 0, ws>>>(P);
            else if (adj) k_photon<Real, false, true><<<gp, bs, 0, ws>>>(P);
            else if (multi) k_photon<Real, true><<<gp, bs, 0, ws>>>(P);
            else k_photon<Real, false><<<gp, bs, 0, ws>>>(P);
            if ((e = cudaGetLastError())) break;
            if (events && (e = cudaEventRecord(gev[4 * r + 1], ws))) break;
            if (events && (e = cudaEventRecord(gev[4 * r + 2], ws))) break;
            if (hfl) k_electron<Real, false, false, true><<<ge, bs, 0, ws>>>(P);
            else if (pi && multi) k_electron<Real, true, false, false, true><<<ge, bs, 0, ws>>>(P);
            else if (pi) k_electron<Real, false, false, false, true><<<ge, bs, 0, ws>>>(P);
            else if (adj) k_electron<Real, false, true><<<ge, bs, 0, ws>>>(P);
            else if (multi) launch_electron<true>(P, ge, bs);
            else launch_electron<false>(P, ge, bs);
            if ((e = cudaGetLastError())) break;
            if (events && (e = cudaEventRecord(gev[4 * r + 3], ws))) break;
        }
        return e;
    }

    // Captures the rounds (without events) into a graph; on any failure the
    // engine keeps launching directly.
    void build_graph(const Params<Real> &P0, int gp, int ge, int bs, bool multi, bool hfl) {
        if (gexec) { cudaGraphExecDestroy(gexec); gexec = nullptr; }
        if (cudaStreamBeginCapture(ws, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            cudaGetLastError();
            graph_ok = false;
            return;
        }
        cudaError_t e = enqueue_rounds(P0, gp, ge, bs, false, multi, false, hfl);
        cudaGraph_t g = nullptr;
        cudaError_t e2 = cudaStreamEndCapture(ws, &g);
        if (e == cudaSuccess && e2 == cudaSuccess && g) e = cudaGraphInstantiate(&gexec, g, 0);
        else if (e == cudaSuccess) e = e2;
        if (g) cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            cudaGetLastError();
            if (gexec) { cudaGraphExecDestroy(gexec); gexec = nullptr; }
            graph_ok = false;
        }
    }

    // Device-side wavefront loop (egsgpu_config.use_graph = 2): a graph whose
    // conditional WHILE node repeats a body of two rounds (queues 0 -> 1 -> 0)
    // and k_rounds, so that one graph launch per chunk transports it to the
    // end without the host looking at the queues in between.  On any failure
    // the engine falls back to launching the rounds directly.
    static constexpr unsigned MAX_ROUNDS = 100000;
    cudaGraphExec_t gexec_loop = nullptr;
    bool loop_ok = true;
    DevMem d_rounds;

    void build_loop_graph(const Params<Real> &P0, int gp, int ge, int bs, bool multi, bool hfl) {
        if (gexec_loop) { cudaGraphExecDestroy(gexec_loop); gexec_loop = nullptr; }
        cudaGraph_t g = nullptr;
        cudaError_t e = d_rounds.alloc(sizeof(unsigned));
        if (e == cudaSuccess) e = cudaGraphCreate(&g, 0);
        cudaGraphConditionalHandle hc = 0;
        if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&hc, g, 1, cudaGraphCondAssignDefault);
        // (the parameter union has no default constructor: zeroed storage)
        alignas(cudaGraphNodeParams) unsigned char np_raw[sizeof(cudaGraphNodeParams)] = {};
        cudaGraphNodeParams &np = *reinterpret_cast<cudaGraphNodeParams *>(np_raw);
        np.type = cudaGraphNodeTypeConditional;
        np.conditional.handle = hc;
        np.conditional.type = cudaGraphCondTypeWhile;
        np.conditional.size = 1;
        cudaGraphNode_t node = nullptr;
        if (e == cudaSuccess) e = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &np);
        bool capturing = false;
        if (e == cudaSuccess) {
            e = cudaStreamBeginCaptureToGraph(ws, np.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                              cudaStreamCaptureModeThreadLocal);
            capturing = e == cudaSuccess;
        }
        if (e == cudaSuccess) e = enqueue_rounds(P0, gp, ge, bs, false, multi, false, hfl, 2);
        if (e == cudaSuccess) {
            k_rounds<<<1, 1, 0, ws>>>(hc, (const unsigned *)d_counts.p, (unsigned *)d_rounds.p, MAX_ROUNDS,
                                      (int *)d_error.p);
            e = cudaGetLastError();
        }
        if (capturing) {
            cudaGraph_t body = nullptr;
            cudaError_t e2 = cudaStreamEndCapture(ws, &body);
            if (e == cudaSuccess) e = e2;
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&gexec_loop, g, 0);
        if (g) cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            cudaGetLastError();
            if (gexec_loop) { cudaGraphExecDestroy(gexec_loop); gexec_loop = nullptr; }
            loop_ok = false;
        }
    }

    float elapsed(cudaEvent_t a, cudaEvent_t b) {
        float ms = 0;
        return cudaEventElapsedTime(&ms, a, b) == cudaSuccess ? ms : 0.f;
    }

    int run(const Source &S, long long first, long long n, int nbatch, uint32_t seed, cudaStream_t st,
            std::string &err) override {
        if (nprob) { err = "the engine holds several phantoms; set one geometry first"; return EGSGPU_ERR_STATE; }
        return run_impl<false>(S, first, n, nbatch, seed, st, err);
    }

    // The device loops' iteration caps of this handle (egsgpu_config.loop_cap,
    // .step_cap), written to the translation unit's constants before a run.
    cudaError_t set_caps(cudaStream_t st) {
        const int caps[2] = {cfg.loop_cap > 0 ? cfg.loop_cap : LOOP_CAP_DEFAULT,
                             cfg.step_cap > 0 ? cfg.step_cap : STEP_CAP_DEFAULT};
        cudaError_t e = cudaMemcpyToSymbolAsync(c_loop_cap, &caps[0], sizeof(int), 0, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyToSymbolAsync(c_step_cap, &caps[1], sizeof(int), 0, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);   // the caps are read from host stack memory
        return e;
    }

    // Histories of batch b of a run of n histories in nbatch batches
    // (the same split for one phantom and for each phantom of many).
    static void batch_range(long long first, long long n, int nbatch, int b, long long &b0, long long &bn) {
        long long per = n / nbatch;
        b0 = first + b * per;
        bn = (b == nbatch - 1) ? n - b * per : per;
    }

    template <bool Multi>
    int run_impl(const Source &S, long long first, long long n, int nbatch, uint32_t seed, cudaStream_t st,
                 std::string &err) {
        if (!G.xb) { err = "geometry not set"; return EGSGPU_ERR_STATE; }
        unsigned cap = cfg.capacity > 0 ? (unsigned)std::min<long long>(cfg.capacity, 0x7fffffffLL) : default_capacity();
        if (int rc = ensure_queues(cap, err)) return rc;
        if (!events_ready) {
            for (auto &e : ev) CK(cudaEventCreate(&e));
            for (auto &e : gev) CK(cudaEventCreate(&e));
            CK(cudaEventCreateWithFlags(&ev_in, cudaEventDisableTiming));
            CK(cudaStreamCreateWithFlags(&ws, cudaStreamNonBlocking));
            events_ready = true;
        }
        // Chunk autotuner: histories per wavefront double while the fullest
        // queue of a chunk stays below a third of its capacity and a doubling
        // does not cost more than 10% of the measured throughput; a queue above
        // two thirds halves the chunk.  Results do not depend on the chunking
        // (every history owns its random-number streams).
        long long chunk = cfg.chunk;
        const bool tune = chunk <= 0;
        if (tune) {
            if (tuned_chunk <= 0) {
                double emax = std::max(S.energy, 0.1);
                double per = (S.charge == 0 ? 12.0 : 16.0) + 8.0 * emax;
                tuned_chunk = std::max<long long>(1024, (long long)(capacity / per));
            }
            chunk = tuned_chunk;
        }
        // persistent grids, one per kernel: never more CTAs than can be
        // resident at once (the photon kernel, with fewer registers, fits more
        // CTAs per SM than the electron kernel)
        const bool adj = mode && mode->adj;
        const bool hfl = cfg.howfarless > 0;
        if (hfl && (Multi || mode)) { err = "HOWFARLESS transport is for one homogeneous phantom (no adjoint)"; return EGSGPU_ERR_ARG; }
        if (hfl && !homogeneous) { err = "HOWFARLESS transport needs a homogeneous phantom"; return EGSGPU_ERR_ARG; }
        const bool pi = cfg.bca_algorithm == 1;
        if (pi && (mode || hfl)) {
            err = "PRESTA-I boundary crossing is for egsgpu_run and egsgpu_run_phantoms (no HOWFARLESS, no adjoint)";
            return EGSGPU_ERR_ARG;
        }
        if (hfl)
            if (int rc = hfl_tables(err)) return rc;
        // The launch shape of candidate k (see SHAPES): threads per CTA and the
        // grids of both kernels.
        int bs = 128, gp = 0, ge = 0;
        auto shape = [&](int k) -> cudaError_t {
            const Shape sh = cfg.block_size > 0 || cfg.ctas_per_sm > 0 ? Shape{cfg.block_size > 0 ? cfg.block_size : 128, 0, 0}
                                                                       : SHAPES[k];
            bs = sh.bs;
            int occ_p = 1, occ_e = 1;
            cudaError_t e;
            if (hfl) {
                e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_p, k_photon<Real, false, false, true>, bs, 0);
                if (!e) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_e, k_electron<Real, false, false, true>, bs, 0);
            } else if (pi) {
                e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_p, k_photon<Real, Multi>, bs, 0);
                if (!e) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_e, k_electron<Real, Multi, false, false, true>, bs, 0);
            } else if (adj) {
                e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_p, k_photon<Real, false, true>, bs, 0);
                if (!e) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_e, k_electron<Real, false, true>, bs, 0);
            } else {
                e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_p, k_photon<Real, Multi>, bs, 0);
                if (!e) e = electron_occupancy<Multi>(occ_e, bs);
            }
            const int cps_cap = cfg.ctas_per_sm > 0 ? cfg.ctas_per_sm : 64;
            gp = sm_count * std::max(1, std::min(cps_cap, occ_p + sh.dp));
            ge = sm_count * std::max(1, std::min(cps_cap, occ_e + sh.de));
            return e;
        };
        // Launch-shape autotuner: once the chunk size has settled, successive
        // chunks of egsgpu_run / egsgpu_run_phantoms try the candidate shapes,
        // and the fastest (by more than 2% over the first) is kept for the
        // engine's later runs.  Only without an explicit block_size or
        // ctas_per_sm, graph replay or adjoint replays; results do not depend
        // on the shape.
        const bool tune_shape = cfg.block_size <= 0 && cfg.ctas_per_sm <= 0 && cfg.use_graph <= 0 && !mode;
        int cur_shape = tune_shape ? (shape_sel >= 0 ? shape_sel : 0) : 0;
        CK(shape(cur_shape));
        Params<Real> P;
        std::memset(&P, 0, sizeof(P));
        P.T = T; P.G = G;
        if (hfl) P.T.etab = (const Real *)d_etab_hfl.p;
        P.dose = (double *)d_dose.p;
        P.hist_tally = (!Multi && hist_n > 0) ? (double *)d_hist.p : nullptr;
        P.hist_first = hist_first; P.hist_n = hist_n;
        P.energy = (double *)d_energy.p;
        P.counters = (unsigned long long *)d_counters.p;
        P.error = (int *)d_error.p;
        P.peak = (unsigned *)d_counts.p + 8;
        P.seed = seed;
        P.requeue_lanes = cfg.requeue_lanes > 0 ? cfg.requeue_lanes : 0;
        P.inter_batch = cfg.inter_batch > 0 ? std::min(cfg.inter_batch, 32) : (cfg.inter_batch < 0 ? 1 : 8);
        P.inter_batch_p = cfg.inter_batch > 0 ? std::min(cfg.inter_batch, 32) : (cfg.inter_batch < 0 ? 1 : 12);
        if (Multi) {
            P.probs = (const Geom<Real> *)d_probs.p; P.pseeds = (const uint32_t *)d_pseeds.p;
            P.psrc = (const Source *)d_psrc.p; P.pvoff = (const int *)d_pvoff.p;
            P.pprefix = (const long long *)d_pprefix.p; P.pfirst = (const long long *)d_pfirst.p;
            P.nprob = nprob;
        }
        if (mode) {   // a replay for the adjoint: its own tallies, never the run's
            P.dose = mode->dose; P.energy = mode->energy; P.counters = mode->counters;
            P.hist_tally = mode->hist; P.hist_first = mode->hist_first; P.hist_n = mode->hist_n;
            P.wvox = mode->wvox; P.hist_G = mode->hist_G; P.grad = mode->grad;
            P.requeue_lanes = 0;
        }
        P.pin = q[0]; P.ein = q[2]; P.pout = q[0]; P.eout = q[2];
        const bool use_graph = cfg.use_graph == 1 && graph_ok && !mode;
        if (use_graph) build_graph(P, gp, ge, bs, Multi, hfl);
        const bool graph = use_graph && gexec;
        const bool use_loop = cfg.use_graph == 2 && loop_ok && !mode;
        if (use_loop) build_loop_graph(P, gp, ge, bs, Multi, hfl);
        const bool looping = use_loop && gexec_loop;
        unsigned *counts = (unsigned *)d_counts.p;
        CK(cudaEventRecord(ev_in, st));
        CK(cudaStreamWaitEvent(ws, ev_in, 0));
        CK(set_caps(ws));
        std::vector<long long> hprefix(nprob + 1), hfirst(nprob + 1);
        for (int b = 0; b < nbatch; ++b) {
            long long b0, bn;
            if (Multi) {
                // batch b of every phantom, laid end to end
                hprefix[0] = 0;
                for (int k = 0; k < nprob; ++k) {
                    long long f, c;
                    batch_range(pdone[k], phist[k], nbatch, b, f, c);
                    hfirst[k] = f;
                    hprefix[k + 1] = hprefix[k] + c;
                }
                hfirst[nprob] = 0;
                CK(cudaMemcpyAsync(d_pprefix.p, hprefix.data(), (nprob + 1) * sizeof(long long), cudaMemcpyHostToDevice, ws));
                CK(cudaMemcpyAsync(d_pfirst.p, hfirst.data(), (nprob + 1) * sizeof(long long), cudaMemcpyHostToDevice, ws));
                b0 = 0;
                bn = hprefix[nprob];
            } else {
                batch_range(first, n, nbatch, b, b0, bn);
            }
            for (long long c0 = b0, cn = 0; c0 < b0 + bn; c0 += cn) {
                cn = std::min(chunk, b0 + bn - c0);   // the autotuner may change `chunk` below
                // shapes are timed on chunks of one size: full chunks once the
                // chunk size has settled, or whole batches smaller than a chunk
                // (never the remainder of a batch)
                const bool whole = (cn == chunk && (!tune || tune_done)) || (c0 == b0 && cn == bn && cn < chunk);
                const bool trying = tune_shape && shape_sel < 0 && whole && (shape_try == 0 || cn == shape_cn);
                if (trying && shape_try == 0) shape_cn = cn;
                if (trying && cur_shape != shape_try) {
                    cur_shape = shape_try;
                    CK(shape(cur_shape));
                }
                auto t_chunk = std::chrono::steady_clock::now();
                CK(cudaMemsetAsync(counts, 0, 9 * sizeof(unsigned), ws));
                CK(cudaEventRecord(ev[0], ws));
                k_source<Real, Multi><<<(unsigned)((cn + 255) / 256), 256, 0, ws>>>(P, S, c0, cn);
                CK(cudaGetLastError());
                CK(cudaEventRecord(ev[1], ws));
                unsigned h[9] = {};
                bool done = false;
                if (looping) {   // one launch runs the chunk's rounds on the device
                    unsigned nr = 0;
                    CK(cudaMemsetAsync(d_rounds.p, 0, sizeof(unsigned), ws));
                    CK(cudaGraphLaunch(gexec_loop, ws));
                    CK(cudaMemcpyAsync(h, counts, sizeof(h), cudaMemcpyDeviceToHost, ws));
                    CK(cudaMemcpyAsync(&nr, d_rounds.p, sizeof(unsigned), cudaMemcpyDeviceToHost, ws));
                    CK(cudaStreamSynchronize(ws));
                    prof_ms[0] += elapsed(ev[0], ev[1]); ++prof_n[0];
                    prof_n[1] += nr; prof_n[2] += nr;
                    if (h[8] > capacity || h[0] > capacity || h[4] > capacity) {
                        err = "particle queue capacity exceeded; lower egsgpu_config.chunk or raise capacity";
                        return EGSGPU_ERR_CAPACITY;
                    }
                    done = (h[0] == 0 && h[4] == 0);
                }
                for (int rep = 0; rep < 100000 / ROUNDS && !done && !looping; ++rep) {
                    if (graph) CK(cudaGraphLaunch(gexec, ws));
                    else CK(enqueue_rounds(P, gp, ge, bs, true, Multi, adj, hfl));
                    CK(cudaMemcpyAsync(h, counts, sizeof(h), cudaMemcpyDeviceToHost, ws));
                    CK(cudaStreamSynchronize(ws));
                    if (rep == 0) { prof_ms[0] += elapsed(ev[0], ev[1]); ++prof_n[0]; }
                    for (int r = 0; r < ROUNDS; ++r) {
                        if (!graph) {
                            prof_ms[1] += elapsed(gev[4 * r], gev[4 * r + 1]);
                            prof_ms[2] += elapsed(gev[4 * r + 2], gev[4 * r + 3]);
                        }
                        ++prof_n[1];
                        ++prof_n[2];
                    }
                    if (h[8] > capacity || h[0] > capacity || h[4] > capacity) {
                        err = "particle queue capacity exceeded; lower egsgpu_config.chunk or raise capacity";
                        return EGSGPU_ERR_CAPACITY;
                    }
                    done = (h[0] == 0 && h[4] == 0);
                }
                if (!done) { err = "wavefront did not drain"; return EGSGPU_ERR_LOOP; }
                if (trying) {
                    const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_chunk).count();
                    shape_rate[shape_try] = cn / std::max(dt, 1e-9);
                    if (++shape_try == NSHAPES) {
                        int best = 0;
                        for (int k = 1; k < NSHAPES; ++k)
                            if (shape_rate[k] > 1.02 * shape_rate[0] && shape_rate[k] > shape_rate[best]) best = k;
                        shape_sel = best;
                        if (cur_shape != best) {
                            cur_shape = best;
                            CK(shape(cur_shape));
                        }
                    }
                }
                if (tune && cn == chunk) {
                    double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_chunk).count();
                    double rate = cn / std::max(dt, 1e-9);
                    unsigned peak = h[8];
                    if (peak > 2 * (capacity / 3)) {
                        tuned_chunk = chunk = std::max<long long>(1024, chunk / 2);
                        tune_done = true;
                    } else if (!tune_done) {
                        if (best_rate > 0 && rate < 0.9 * best_rate) {
                            tuned_chunk = chunk = best_chunk;
                            tune_done = true;
                        } else {
                            if (rate > best_rate) { best_rate = rate; best_chunk = chunk; }
                            if (peak < capacity / 3 && chunk < (1LL << 30)) tuned_chunk = chunk = chunk * 2;
                            else tune_done = true;
                        }
                    }
                }
            }
            if (mode) { CK(cudaStreamSynchronize(ws)); continue; }
            CK(cudaEventRecord(ev[6], ws));
            k_batch<<<std::max(1, std::min(4 * sm_count, (int)((nvox + 255) / 256))), 256, 0, ws>>>(
                (double *)d_dose.p, (double *)d_sum.p, (double *)d_sum2.p, nvox);
            CK(cudaGetLastError());
            CK(cudaEventRecord(ev[7], ws));
            CK(cudaStreamSynchronize(ws));
            prof_ms[3] += elapsed(ev[6], ev[7]);
            ++prof_n[3];
        }
        CK(cudaStreamSynchronize(ws));
        int e[2];
        CK(cudaMemcpy(e, d_error.p, sizeof(e), cudaMemcpyDeviceToHost));
        if (e[0]) { err = "particle queue capacity exceeded"; return EGSGPU_ERR_CAPACITY; }
        if (e[1]) { err = "a device sampling loop hit its iteration cap"; return EGSGPU_ERR_LOOP; }
        return 0;
    }

    // ------------------------------------------------------- adjoint ----
    // A replay of histories for the adjoint writes to scratch tallies, so the
    // run being differentiated keeps its own.
    struct RunMode {
        bool adj;
        double *dose, *energy;
        unsigned long long *counters;
        double *hist;
        long long hist_first, hist_n;
        const double *wvox, *hist_G;
        double *grad;
    };
    const RunMode *mode = nullptr;
    DevMem d_aw, d_agrad, d_aG, d_adose, d_aenergy, d_acount;

    // dL/d(rhor) of the histories [first, first+n) for energy weights
    // w_v = dL/dE_v: pass 1 replays the histories with weighted per-history
    // tallies (G_h = sum of w_v * deposit over history h), pass 2 replays them
    // again with the adjoint kernels, which add the photon path scores times
    // G_h and the electrons' pathwise continuous-loss terms.
    int adjoint(const Source &S, long long first, long long n, uint32_t seed, const double *w, double *grad,
                std::string &err) override {
        if (!G.xb || nprob) { err = "a single geometry must be set"; return EGSGPU_ERR_STATE; }
        CK(d_aw.alloc(nvox * sizeof(double)));
        CK(d_agrad.alloc(nvox * sizeof(double)));
        CK(d_aG.alloc(n * sizeof(double)));
        CK(d_adose.alloc(nvox * sizeof(double)));
        CK(d_aenergy.alloc(2 * sizeof(double)));
        CK(d_acount.alloc(CNT_N * sizeof(unsigned long long)));
        CK(cudaMemcpy(d_aw.p, w, nvox * sizeof(double), cudaMemcpyHostToDevice));
        CK(cudaMemset(d_agrad.p, 0, nvox * sizeof(double)));
        CK(cudaMemset(d_aG.p, 0, n * sizeof(double)));
        CK(cudaMemset(d_adose.p, 0, nvox * sizeof(double)));
        CK(cudaMemset(d_aenergy.p, 0, 2 * sizeof(double)));
        CK(cudaMemset(d_acount.p, 0, CNT_N * sizeof(unsigned long long)));
        RunMode m{false, (double *)d_adose.p, (double *)d_aenergy.p, (unsigned long long *)d_acount.p,
                  (double *)d_aG.p, first, n, (const double *)d_aw.p, nullptr, nullptr};
        mode = &m;
        int rc = run_impl<false>(S, first, n, 1, seed, nullptr, err);
        if (!rc) {
            m = RunMode{true, (double *)d_adose.p, (double *)d_aenergy.p, (unsigned long long *)d_acount.p,
                        nullptr, first, n, (const double *)d_aw.p, (const double *)d_aG.p, (double *)d_agrad.p};
            rc = run_impl<false>(S, first, n, 1, seed, nullptr, err);
        }
        mode = nullptr;
        if (rc) return rc;
        CK(cudaMemcpy(grad, d_agrad.p, nvox * sizeof(double), cudaMemcpyDeviceToHost));
        return 0;
    }

    // ------------------------------------------------ several phantoms ----
    // The phantoms' planes, media and densities are laid end to end in the
    // engine's geometry buffers (phantom k's voxels at global indices
    // [voff_k, voff_k+1)), so the tallies, the batch fold and the read-back
    // serve all phantoms at once.
    int nprob = 0;
    std::vector<long long> phist;   // histories per phantom per run
    std::vector<long long> pdone;   // histories already transported per phantom
    DevMem d_probs, d_pseeds, d_psrc, d_pvoff, d_pprefix, d_pfirst;

    int problems(int n, const PhantomDesc *pd, const Source *src, std::string &err) override {
        std::vector<Real> x, y, z;
        raw_vector<Real> r;
        raw_vector<uint8_t> m;
        std::vector<int> voff(n + 1, 0);
        std::vector<long long> xo(n), yo(n), zo(n);
        long long tot = 0;
        for (int k = 0; k < n; ++k) {
            const PhantomDesc &d = pd[k];
            long long nv = (long long)d.nx * d.ny * d.nz;
            if (tot + nv > 0x7fffffffLL) { err = "too many voxels over all phantoms"; return EGSGPU_ERR_ARG; }
            voff[k] = (int)tot;
            xo[k] = (long long)x.size(); yo[k] = (long long)y.size(); zo[k] = (long long)z.size();
            x.insert(x.end(), d.xb, d.xb + d.nx + 1);
            y.insert(y.end(), d.yb, d.yb + d.ny + 1);
            z.insert(z.end(), d.zb, d.zb + d.nz + 1);
            tot += nv;
        }
        voff[n] = (int)tot;
        // voxels of all phantoms end to end, converted over the global index
        m.resize(tot);
        r.resize(tot);
        const std::vector<long long> off(voff.begin(), voff.end());
        phantoms_parallel(off, [&](int k, long long b, long long e) {
            uint8_t *mo = m.data() + off[k];
            Real *ro = r.data() + off[k];
            for (long long i = b; i < e; ++i) { mo[i] = (uint8_t)pd[k].med[i]; ro[i] = (Real)pd[k].rhor[i]; }
        });
        auto up = [&](DevMem &dm, const void *p, size_t bytes) -> cudaError_t {
            cudaError_t e = dm.alloc(bytes);
            if (e != cudaSuccess) return e;
            return cudaMemcpy(dm.p, p, bytes, cudaMemcpyHostToDevice);
        };
        CK(up(d_xb, x.data(), x.size() * sizeof(Real)));
        CK(up(d_yb, y.data(), y.size() * sizeof(Real)));
        CK(up(d_zb, z.data(), z.size() * sizeof(Real)));
        CK(up(d_med, m.data(), m.size()));
        CK(up(d_rhor, r.data(), r.size() * sizeof(Real)));
        const Real bt = sizeof(Real) == 8 ? (Real)(1.0 / 4294967296.0) : (Real)(1.0 / 2097152.0);
        std::vector<Geom<Real>> gs(n);
        std::vector<uint32_t> seeds(n);
        phist.assign(n, 0);
        for (int k = 0; k < n; ++k) {
            Geom<Real> &g = gs[k];
            g.nx = pd[k].nx; g.ny = pd[k].ny; g.nz = pd[k].nz; g.nxy = g.nx * g.ny;
            g.xb = (const Real *)d_xb.p + xo[k]; g.yb = (const Real *)d_yb.p + yo[k]; g.zb = (const Real *)d_zb.p + zo[k];
            g.med = (const uint8_t *)d_med.p; g.rhor = (const Real *)d_rhor.p;
            g.bt = bt; g.hbt = bt / 2;
            g.voff = voff[k];
            set_divisors(g);
            seeds[k] = pd[k].seed;
            phist[k] = pd[k].histories;
        }
        CK(up(d_probs, gs.data(), n * sizeof(Geom<Real>)));
        CK(up(d_pseeds, seeds.data(), n * sizeof(uint32_t)));
        CK(up(d_psrc, src, n * sizeof(Source)));
        CK(up(d_pvoff, voff.data(), (n + 1) * sizeof(int)));
        CK(d_pprefix.alloc((n + 1) * sizeof(long long)));
        CK(d_pfirst.alloc((n + 1) * sizeof(long long)));
        G = gs[0];
        nvox = tot;
        nprob = n;
        homogeneous = false;
        pdone.assign(n, 0);
        CK(d_dose.alloc(nvox * sizeof(double)));
        CK(d_sum.alloc(nvox * sizeof(double)));
        CK(d_sum2.alloc(nvox * sizeof(double)));
        CK(cudaMemset(d_dose.p, 0, nvox * sizeof(double)));
        CK(cudaMemset(d_sum.p, 0, nvox * sizeof(double)));
        CK(cudaMemset(d_sum2.p, 0, nvox * sizeof(double)));
        return 0;
    }

    // Each call transports the next histories of every phantom: the first
    // call histories [0, n_k), the second [n_k, 2 n_k), ...
    int run_multi(const Source &Smax, int nbatch, cudaStream_t st, std::string &err) override {
        if (!nprob) { err = "no phantoms set"; return EGSGPU_ERR_STATE; }
        for (int k = 0; k < nprob; ++k)
            if (pdone[k] + phist[k] > 0xffffffffLL) { err = "history index beyond 2^32"; return EGSGPU_ERR_ARG; }
        int rc = run_impl<true>(Smax, 0, 0, nbatch, 0, st, err);
        if (!rc)
            for (int k = 0; k < nprob; ++k) pdone[k] += phist[k];
        return rc;
    }

    // Transport of one small chunk with every piece of scratch (queues,
    // counters, error flags) carved out of a caller-independent static device
    // array; all work goes to the caller's stream.  See egsgpu_run_noalloc.
    int run_noalloc(const Source &S, long long first, long long n, uint32_t seed, double *dose, cudaStream_t st,
                    unsigned char *scratch, size_t scratch_bytes, std::string &err) override {
        if (!G.xb || nprob) { err = "a single geometry must be set"; return EGSGPU_ERR_STATE; }
        // layout: 1 KiB of counters, then four queues of equal capacity
        unsigned *counts = (unsigned *)scratch;                          // 16 x unsigned
        double *energy = (double *)(scratch + 256);                      // 2 x double
        unsigned long long *counters = (unsigned long long *)(scratch + 512);   // CNT_N
        int *error = (int *)(scratch + 896);                             // 2 x int
        const size_t rec = 12 * sizeof(Real) + sizeof(int) + 2 + 2 * sizeof(uint32_t) + sizeof(unsigned long long);
        size_t avail = scratch_bytes - 1024 - 4 * 16 * 256;
        unsigned cap = (unsigned)((avail / (4 * rec)) & ~(size_t)255);
        Queue<Real> Q[4];
        unsigned char *b = scratch + 1024;
        auto take = [&](size_t bytes) { unsigned char *r = b; b += (bytes + 255) & ~(size_t)255; return r; };
        for (int k = 0; k < 4; ++k) {
            Queue<Real> &q = Q[k];
            q.x = (Real *)take(cap * sizeof(Real)); q.y = (Real *)take(cap * sizeof(Real));
            q.z = (Real *)take(cap * sizeof(Real)); q.u = (Real *)take(cap * sizeof(Real));
            q.v = (Real *)take(cap * sizeof(Real)); q.w = (Real *)take(cap * sizeof(Real));
            q.E = (Real *)take(cap * sizeof(Real)); q.wt = (Real *)take(cap * sizeof(Real));
            q.ir = (int *)take(cap * sizeof(int)); q.iq = (int8_t *)take(cap);
            q.hist = (uint32_t *)take(cap * sizeof(uint32_t)); q.n = (uint32_t *)take(cap * sizeof(uint32_t));
            q.sid = (unsigned long long *)take(cap * sizeof(unsigned long long));
            q.st = (uint8_t *)take(cap);
            q.aux0 = (Real *)take(cap * sizeof(Real)); q.aux1 = (Real *)take(cap * sizeof(Real));
            q.aux2 = (Real *)take(cap * sizeof(Real)); q.aux3 = (Real *)take(cap * sizeof(Real));
            q.count = counts + 2 * k;
            q.capacity = cap;
        }
        if ((size_t)(b - scratch) > scratch_bytes) { err = "no-allocation scratch layout overflow"; return EGSGPU_ERR_STATE; }
        // launch shapes and interaction batching as egsgpu_run takes them
        const int bs = cfg.block_size > 0 ? cfg.block_size : 128;
        int occ_p = 1, occ_e = 1;
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_p, k_photon<Real, false>, bs, 0));
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_e, k_electron<Real, false>, bs, 0));
        const int cps_cap = cfg.ctas_per_sm > 0 ? cfg.ctas_per_sm : 64;
        const int gp = sm_count * std::max(1, std::min(cps_cap, occ_p));
        const int ge = sm_count * std::max(1, std::min(cps_cap, occ_e));
        Params<Real> P;
        std::memset(&P, 0, sizeof(P));
        P.T = T; P.G = G;
        P.dose = dose;
        P.hist_tally = nullptr; P.hist_first = 0; P.hist_n = 0;
        P.energy = energy; P.counters = counters; P.error = error; P.peak = counts + 8;
        P.seed = seed;
        P.requeue_lanes = 0;
        P.inter_batch = cfg.inter_batch > 0 ? std::min(cfg.inter_batch, 32) : (cfg.inter_batch < 0 ? 1 : 8);
        P.inter_batch_p = cfg.inter_batch > 0 ? std::min(cfg.inter_batch, 32) : (cfg.inter_batch < 0 ? 1 : 12);
        // the array keeps the previous call's contents: clear the counters
        CK(cudaMemsetAsync(scratch, 0, 1024, st));
        CK(set_caps(st));
        CK(cudaMemsetAsync(dose, 0, (size_t)nvox * sizeof(double), st));
        P.pout = Q[0]; P.eout = Q[2]; P.pin = Q[0]; P.ein = Q[2];
        k_source<Real, false><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(P, S, first, n);
        CK(cudaGetLastError());
        int cur = 0;
        bool done = false;
        for (int round = 0; round < 100000 && !done; ++round) {
            int nxt = 1 - cur;
            CK(cudaMemsetAsync(counts + 2 * nxt, 0, 2 * sizeof(unsigned), st));
            CK(cudaMemsetAsync(counts + 4 + 2 * nxt, 0, 2 * sizeof(unsigned), st));
            P.pin = Q[cur]; P.ein = Q[2 + cur]; P.pout = Q[nxt]; P.eout = Q[2 + nxt];
            k_photon<Real, false><<<gp, bs, 0, st>>>(P);
            CK(cudaGetLastError());
            k_electron<Real, false><<<ge, bs, 0, st>>>(P);
            CK(cudaGetLastError());
            unsigned h[9];
            CK(cudaMemcpyAsync(h, counts, sizeof(h), cudaMemcpyDeviceToHost, st));
            CK(cudaStreamSynchronize(st));
            if (h[8] > cap) { err = "no-allocation scratch queues overflowed; transport fewer histories per call"; return EGSGPU_ERR_CAPACITY; }
            cur = nxt;
            done = h[2 * cur] == 0 && h[4 + 2 * cur] == 0;
        }
        if (!done) { err = "wavefront did not drain"; return EGSGPU_ERR_LOOP; }
        int e[2];
        CK(cudaMemcpyAsync(e, error, sizeof(e), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        if (e[0]) { err = "no-allocation scratch queues overflowed"; return EGSGPU_ERR_CAPACITY; }
        if (e[1]) { err = "a device sampling loop hit its iteration cap"; return EGSGPU_ERR_LOOP; }
        return 0;
    }
};

}  // namespace EGSGPU_TU
}  // namespace egsgpu_host

using namespace egsgpu_host;
using namespace egsgpu_host::EGSGPU_TU;

#ifdef EGSGPU_PART_F64
// The FP64 translation unit contributes its engine only.
EngineBase *egsgpu_host::make_engine_f64(const egsgpu_config &c) { return new Engine<double>(c); }
#else

struct egsgpu_handle {
    egsgpu_config cfg;
    std::string err;
    egs::Hatch H;
    bool have_media = false, have_geom = false, have_source = false;
    std::unique_ptr<EngineBase> eng;
    // geometry copies for dose normalisation
    int nx = 0, ny = 0, nz = 0;
    std::vector<double> xb, yb, zb;
    raw_vector<double> rhor;
    raw_vector<int32_t> med;
    // source
    Source S{};
    DevMem d_edges, d_wi, d_bin, d_phsp;
    long long nhist = 0;
    int nbatch = 0;
    double ecut = 0, pcut = 0;
    // several phantoms (egsgpu_set_phantoms): host copies for the dose
    // normalisation, global voxel offsets, histories run per phantom
    struct Phantom {
        int nx, ny, nz;
        std::vector<double> xb, yb, zb;
        raw_vector<double> rhor;
        raw_vector<int32_t> med;
        long long voff, histories, nhist;
    };
    std::vector<Phantom> phantoms;
    long long mvox = 0;
    Source Smax{};
    DevMem d_pedges, d_pwi, d_pbin, d_pphsp;
    bool multi() const { return !phantoms.empty(); }
    long long nvox() const { return multi() ? mvox : (long long)nx * ny * nz; }
};

static int get_tallies_impl(egsgpu_handle *h, double *sum, double *sum2, double *totals) {
    long long nv = h->nvox();
    if (int rc = h->eng->read_sums(0, nv, sum, sum2, h->err)) return rc;
    if (totals) {
        double en[2];
        unsigned long long c[CNT_N];
        if (int rc = h->eng->read_totals(en, c, h->err)) return rc;
        totals[0] = (double)h->nhist; totals[1] = h->nbatch; totals[2] = en[0]; totals[3] = en[1];
        totals[4] = (double)(c[CNT_PSTEP] + c[CNT_ESTEP]); totals[5] = (double)c[CNT_PSTEP];
        totals[6] = (double)c[CNT_ESTEP]; totals[7] = (double)(c[CNT_PUSH] + c[CNT_EPUSH]);
    }
    return 0;
}

extern "C" {

void egsgpu_default_config(egsgpu_config *c) {
    std::memset(c, 0, sizeof(*c));
    c->ecut = 0.521; c->pcut = 0.010;
    c->estepe = 0.25; c->ximax = 0.5; c->skindepth = 3.0;
    c->precision = 32;
}

int egsgpu_create(const egsgpu_config *cfg, egsgpu_handle **out) {
    if (!cfg || !out) return EGSGPU_ERR_ARG;
    *out = nullptr;
    if (cfg->precision != 32 && cfg->precision != 64) return EGSGPU_ERR_ARG;
    // the transport kernels are compiled for at most MAX_BLOCK threads per CTA
    if (cfg->block_size < 0 || cfg->block_size > MAX_BLOCK || cfg->block_size % 32) return EGSGPU_ERR_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return EGSGPU_ERR_CUDA;
    auto *h = new egsgpu_handle();
    h->cfg = *cfg;
    if (cfg->precision == 32) h->eng.reset(new Engine<float>(*cfg));
    else h->eng.reset(make_engine_f64(*cfg));
    *out = h;
    return 0;
}

int egsgpu_load_media(egsgpu_handle *h, const char *data_dir, const char *pegs_file, const char *const *names,
                      int n) {
    if (!h || !data_dir || !pegs_file || !names || n < 1) return EGSGPU_ERR_ARG;
    egs::TransportParams tp;
    tp.ecut = h->cfg.ecut; tp.pcut = h->cfg.pcut;
    tp.estepe = h->cfg.estepe; tp.ximax = h->cfg.ximax; tp.skindepth_for_bca = h->cfg.skindepth;
    if (h->cfg.smax > 0) tp.smaxir = h->cfg.smax;
    if (h->cfg.bca_algorithm != 0 && h->cfg.bca_algorithm != 1) { h->err = "bca_algorithm must be 0 (EXACT) or 1 (PRESTA-I)"; return EGSGPU_ERR_ARG; }
    tp.exact_bca = h->cfg.bca_algorithm == 0;
    std::vector<std::string> nm;
    for (int i = 0; i < n; ++i) nm.push_back(names[i]);
    int rc = egs::hatch(data_dir, pegs_file, nm, tp, h->H, h->err);
    if (rc) return rc;
    // $adjust_rhor_ecut_pcut: cut-offs not below any AE / AP
    double ecut = h->cfg.ecut, pcut = h->cfg.pcut;
    for (auto &m : h->H.media) { ecut = std::max(ecut, m.ae); pcut = std::max(pcut, m.ap); }
    // Relaxation products are deposited locally: exact only while every shell
    // binding energy is below both transport cut-offs.
    if (h->H.max_binding_energy > std::min(pcut, ecut - egs::RM)) {
        h->err = "a shell binding energy exceeds the cut-offs: relaxation cascades above cut-off are not supported";
        return EGSGPU_ERR_ARG;
    }
    h->ecut = ecut; h->pcut = pcut;
    rc = h->eng->load(h->H, ecut, pcut, h->H.params.skindepth_for_bca, tp.smaxir, h->err);
    if (rc) return rc;
    h->have_media = true;
    return 0;
}

int egsgpu_get_medium(egsgpu_handle *h, int index, double *out) {
    if (!h || !out) return EGSGPU_ERR_ARG;
    if (!h->have_media) { h->err = "no media loaded"; return EGSGPU_ERR_STATE; }
    if (index < 0 || index >= (int)h->H.media.size()) { h->err = "medium index out of range"; return EGSGPU_ERR_ARG; }
    const egs::Medium &m = h->H.media[index];
    out[0] = m.rho; out[1] = m.ae; out[2] = m.ap; out[3] = m.nne;
    return 0;
}

int egsgpu_set_xyz_geometry(egsgpu_handle *h, int nx, int ny, int nz, const double *xb, const double *yb,
                            const double *zb, const int32_t *med, const double *rhor) {
    if (!h || nx < 1 || ny < 1 || nz < 1 || !xb || !yb || !zb || !med || !rhor) return EGSGPU_ERR_ARG;
    if (!h->have_media) { h->err = "load media before the geometry"; return EGSGPU_ERR_STATE; }
    long long nv = (long long)nx * ny * nz;
    if (nv > (1LL << 31) - 1) { h->err = "too many voxels"; return EGSGPU_ERR_ARG; }
    for (int i = 0; i < nx; ++i) if (!(xb[i + 1] > xb[i])) { h->err = "x-planes not increasing"; return EGSGPU_ERR_ARG; }
    for (int i = 0; i < ny; ++i) if (!(yb[i + 1] > yb[i])) { h->err = "y-planes not increasing"; return EGSGPU_ERR_ARG; }
    for (int i = 0; i < nz; ++i) if (!(zb[i + 1] > zb[i])) { h->err = "z-planes not increasing"; return EGSGPU_ERR_ARG; }
    int nmed = (int)h->H.media.size();
    if (int bad = check_voxels(nv, med, rhor, nmed)) {
        h->err = bad == 1 ? "voxel medium index out of range" : "voxel relative density must be positive and finite";
        return EGSGPU_ERR_ARG;
    }
    int rc = h->eng->geometry(nx, ny, nz, xb, yb, zb, med, rhor, h->err);
    if (rc) return rc;
    h->nx = nx; h->ny = ny; h->nz = nz;
    h->xb.assign(xb, xb + nx + 1); h->yb.assign(yb, yb + ny + 1); h->zb.assign(zb, zb + nz + 1);
    h->med.resize(nv); h->rhor.resize(nv);
    host_parallel(nv, [&](long long b, long long e) {
        std::copy(med + b, med + e, h->med.begin() + b);
        std::copy(rhor + b, rhor + e, h->rhor.begin() + b);
    });
    h->have_geom = true;
    h->phantoms.clear();
    h->nhist = 0; h->nbatch = 0;
    return 0;
}

}  // extern "C"

// Checks a source description and builds its host form; a histogram spectrum
// becomes a Walker alias table over its bins (egs++/egs_alias_table.cpp:117-263)
// returned in edges / wi / bin (device pointers are filled in by the caller).
static int build_source(const egsgpu_source *s, Source &S, std::vector<double> &edges, std::vector<double> &wi,
                        std::vector<int> &bin, std::string &err) {
    if (s->charge < -1 || s->charge > 1 || s->shape < 0 || s->shape > 2 || (s->spectrum != 0 && s->spectrum != 1)) {
        err = "unsupported source";
        return EGSGPU_ERR_ARG;
    }
    bool has_rot = false;
    for (double r : s->rot) has_rot |= r != 0;
    if (has_rot && s->shape != 2) { err = "a source rotation is supported for phase-space sources only"; return EGSGPU_ERR_ARG; }
    if (has_rot) {   // R R^T = 1 and det R = +1 to 1e-6
        const double *R = s->rot;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                double d = R[3 * i] * R[3 * j] + R[3 * i + 1] * R[3 * j + 1] + R[3 * i + 2] * R[3 * j + 2];
                if (!(std::fabs(d - (i == j)) < 1e-6)) { err = "the source rotation is not a rotation"; return EGSGPU_ERR_ARG; }
            }
        double det = R[0] * (R[4] * R[8] - R[5] * R[7]) - R[1] * (R[3] * R[8] - R[5] * R[6]) +
                     R[2] * (R[3] * R[7] - R[4] * R[6]);
        if (!(std::fabs(det - 1) < 1e-6)) { err = "the source rotation is not a rotation"; return EGSGPU_ERR_ARG; }
    }
    if (s->shape == 2) {   // phase-space particles: checked here, copied by the caller
        if (s->nphsp < 1 || !s->phsp || s->recycle < 0) { err = "bad phase-space source"; return EGSGPU_ERR_ARG; }
        S = Source{};
        S.shape = 2;
        for (int k = 0; k < 3; ++k) S.pos[k] = s->pos[k];
        S.dir[2] = 1;
        S.nphsp = s->nphsp;
        S.recycle = s->recycle;
        S.has_rot = has_rot;
        for (int k = 0; k < 9; ++k) S.rot[k] = s->rot[k];
        double emax = 0;
        for (long long i = 0; i < s->nphsp; ++i) {
            const float *q = s->phsp + 7 * i;
            if (!(q[0] == -1.0f || q[0] == 0.0f || q[0] == 1.0f) || !(q[1] > 0) || !std::isfinite(q[1]) ||
                !(q[4] * q[4] + q[5] * q[5] <= 1.0f + 1e-5f)) {
                err = "bad phase-space particle " + std::to_string(i);
                return EGSGPU_ERR_ARG;
            }
            emax = std::max(emax, (double)q[1]);
            if (q[0] != 0) S.charge = -1;
        }
        S.energy = emax;
        edges.clear(); wi.clear(); bin.clear();
        return 0;
    }
    double nrm = std::sqrt(s->dir[0] * s->dir[0] + s->dir[1] * s->dir[1] + s->dir[2] * s->dir[2]);
    if (!(nrm > 0)) { err = "zero source direction"; return EGSGPU_ERR_ARG; }
    S = Source{};
    S.charge = s->charge; S.shape = s->shape; S.spectrum = s->spectrum;
    for (int k = 0; k < 3; ++k) { S.pos[k] = s->pos[k]; S.dir[k] = s->dir[k] / nrm; }
    S.xmin = s->xmin; S.xmax = s->xmax; S.ymin = s->ymin; S.ymax = s->ymax;
    S.energy = s->energy;
    edges.clear(); wi.clear(); bin.clear();
    if (s->spectrum == 0) {
        if (!(s->energy > 0)) { err = "source energy must be positive"; return EGSGPU_ERR_ARG; }
        return 0;
    }
    int nb = s->nbins;
    if (nb < 1 || !s->edges || !s->weights) { err = "bad spectrum"; return EGSGPU_ERR_ARG; }
    std::vector<double> w(nb);
    wi.assign(nb, 1.0);
    bin.assign(nb, 0);
    double sum = 0;
    for (int i = 0; i < nb; ++i) {
        if (!(s->edges[i + 1] > s->edges[i]) || s->weights[i] < 0) { err = "bad spectrum bins"; return EGSGPU_ERR_ARG; }
        w[i] = s->weights[i] * (s->edges[i + 1] - s->edges[i]);
        sum += w[i];
    }
    if (!(sum > 0)) { err = "empty spectrum"; return EGSGPU_ERR_ARG; }
    for (int i = 0; i < nb; ++i) w[i] = w[i] / sum * nb;
    std::vector<int> small, large;
    for (int i = 0; i < nb; ++i) (w[i] < 1 ? small : large).push_back(i);
    while (!small.empty() && !large.empty()) {
        int sm = small.back(); small.pop_back();
        int lg = large.back();
        wi[sm] = w[sm]; bin[sm] = lg;
        w[lg] -= 1 - w[sm];
        if (w[lg] < 1) { large.pop_back(); small.push_back(lg); }
    }
    for (int i : small) { wi[i] = 1; bin[i] = i; }
    for (int i : large) { wi[i] = 1; bin[i] = i; }
    edges.assign(s->edges, s->edges + nb + 1);
    S.nbins = nb;
    return 0;
}

extern "C" {

int egsgpu_set_source(egsgpu_handle *h, const egsgpu_source *s) {
    if (!h || !s) return EGSGPU_ERR_ARG;
    Source S;
    std::vector<double> edges, wi;
    std::vector<int> bin;
    if (int rc = build_source(s, S, edges, wi, bin, h->err)) return rc;
    if (s->shape == 2) {
        std::string &err = h->err;
        CK(h->d_phsp.alloc((size_t)s->nphsp * 7 * sizeof(float)));
        CK(cudaMemcpy(h->d_phsp.p, s->phsp, (size_t)s->nphsp * 7 * sizeof(float), cudaMemcpyHostToDevice));
        S.phsp = (const float *)h->d_phsp.p;
    } else if (s->spectrum == 1) {
        std::string &err = h->err;
        int nb = S.nbins;
        CK(h->d_edges.alloc((nb + 1) * sizeof(double)));
        CK(h->d_wi.alloc(nb * sizeof(double)));
        CK(h->d_bin.alloc(nb * sizeof(int)));
        CK(cudaMemcpy(h->d_edges.p, edges.data(), (nb + 1) * sizeof(double), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(h->d_wi.p, wi.data(), nb * sizeof(double), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(h->d_bin.p, bin.data(), nb * sizeof(int), cudaMemcpyHostToDevice));
        S.edges = (const double *)h->d_edges.p; S.wi = (const double *)h->d_wi.p; S.bin = (const int *)h->d_bin.p;
    }
    h->S = S;
    h->have_source = true;
    return 0;
}

int egsgpu_run(egsgpu_handle *h, long long first, long long n, int n_batch, uint32_t seed, void *stream) {
    if (!h || n < 0 || n_batch < 1 || first < 0 || first + n > 0xffffffffLL) return EGSGPU_ERR_ARG;
    if (!h->have_media || !h->have_geom || !h->have_source) { h->err = "media, geometry and source must be set"; return EGSGPU_ERR_STATE; }
    if (n == 0) return 0;
    if (n_batch > n) n_batch = (int)n;
    int rc = h->eng->run(h->S, first, n, n_batch, seed, (cudaStream_t)stream, h->err);
    if (rc) return rc;
    h->nhist += n;
    h->nbatch += n_batch;
    return 0;
}

int egsgpu_set_phantoms(egsgpu_handle *h, int n, const egsgpu_phantom *ph) {
    if (!h || n < 1 || !ph) return EGSGPU_ERR_ARG;
    if (!h->have_media) { h->err = "load media before the phantoms"; return EGSGPU_ERR_STATE; }
    const int nmed = (int)h->H.media.size();
    std::vector<PhantomDesc> pd(n);
    std::vector<Source> src(n);
    std::vector<double> alle, allw;
    std::vector<int> allb;
    std::vector<long long> so(n, -1), bo(n, -1), po(n, -1);
    long long nphsp_all = 0;
    Source smax{};
    long long tot = 0;
    for (int k = 0; k < n; ++k) {
        const egsgpu_phantom &q = ph[k];
        const std::string at = " (phantom " + std::to_string(k) + ")";
        if (q.nx < 1 || q.ny < 1 || q.nz < 1 || !q.xb || !q.yb || !q.zb || !q.med || !q.rhor) {
            h->err = "bad phantom geometry" + at;
            return EGSGPU_ERR_ARG;
        }
        if (q.histories < 0 || q.histories > 0xffffffffLL) { h->err = "bad history count" + at; return EGSGPU_ERR_ARG; }
        long long nv = (long long)q.nx * q.ny * q.nz;
        if (tot + nv > (1LL << 31) - 1) { h->err = "too many voxels over all phantoms"; return EGSGPU_ERR_ARG; }
        tot += nv;
        for (int i = 0; i < q.nx; ++i) if (!(q.xb[i + 1] > q.xb[i])) { h->err = "x-planes not increasing" + at; return EGSGPU_ERR_ARG; }
        for (int i = 0; i < q.ny; ++i) if (!(q.yb[i + 1] > q.yb[i])) { h->err = "y-planes not increasing" + at; return EGSGPU_ERR_ARG; }
        for (int i = 0; i < q.nz; ++i) if (!(q.zb[i + 1] > q.zb[i])) { h->err = "z-planes not increasing" + at; return EGSGPU_ERR_ARG; }
        std::vector<double> e, w;
        std::vector<int> b;
        if (int rc = build_source(&q.source, src[k], e, w, b, h->err)) { h->err += at; return rc; }
        double emax = q.source.energy;
        if (q.source.shape == 2) {
            po[k] = nphsp_all;
            nphsp_all += q.source.nphsp;
            emax = src[k].energy;
        } else if (q.source.spectrum == 1) {
            so[k] = (long long)allw.size();
            bo[k] = (long long)alle.size();
            alle.insert(alle.end(), e.begin(), e.end());
            allw.insert(allw.end(), w.begin(), w.end());
            allb.insert(allb.end(), b.begin(), b.end());
            emax = e.back();
        }
        smax.energy = std::max(smax.energy, emax);
        if (src[k].charge != 0) smax.charge = -1;
        pd[k] = PhantomDesc{q.nx, q.ny, q.nz, q.xb, q.yb, q.zb, q.med, q.rhor, q.seed, q.histories};
    }
    // the voxels of all phantoms, checked in one pass over host threads
    std::vector<long long> off(n + 1, 0);
    for (int k = 0; k < n; ++k) off[k + 1] = off[k] + (long long)ph[k].nx * ph[k].ny * ph[k].nz;
    std::vector<std::atomic<int>> bad(n);
    for (auto &b : bad) b.store(0);
    phantoms_parallel(off, [&](int k, long long b, long long e) {
        if (int v = check_range(e - b, ph[k].med + b, ph[k].rhor + b, nmed)) bad[k].fetch_or(v);
    });
    for (int k = 0; k < n; ++k)
        if (int v = bad[k].load()) {
            h->err = std::string((v & 1) ? "voxel medium index out of range" : "bad voxel relative density") +
                     " (phantom " + std::to_string(k) + ")";
            return EGSGPU_ERR_ARG;
        }
    std::string &err = h->err;
    if (nphsp_all > 0) {
        CK(h->d_pphsp.alloc((size_t)nphsp_all * 7 * sizeof(float)));
        for (int k = 0; k < n; ++k) {
            if (po[k] < 0) continue;
            CK(cudaMemcpy((float *)h->d_pphsp.p + 7 * po[k], ph[k].source.phsp,
                          (size_t)ph[k].source.nphsp * 7 * sizeof(float), cudaMemcpyHostToDevice));
            src[k].phsp = (const float *)h->d_pphsp.p + 7 * po[k];
        }
    }
    if (!allw.empty()) {
        CK(h->d_pedges.alloc(alle.size() * sizeof(double)));
        CK(h->d_pwi.alloc(allw.size() * sizeof(double)));
        CK(h->d_pbin.alloc(allb.size() * sizeof(int)));
        CK(cudaMemcpy(h->d_pedges.p, alle.data(), alle.size() * sizeof(double), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(h->d_pwi.p, allw.data(), allw.size() * sizeof(double), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(h->d_pbin.p, allb.data(), allb.size() * sizeof(int), cudaMemcpyHostToDevice));
        for (int k = 0; k < n; ++k) {
            if (so[k] < 0) continue;
            src[k].edges = (const double *)h->d_pedges.p + bo[k];
            src[k].wi = (const double *)h->d_pwi.p + so[k];
            src[k].bin = (const int *)h->d_pbin.p + so[k];
        }
    }
    int rc = h->eng->problems(n, pd.data(), src.data(), h->err);
    if (rc) { h->phantoms.clear(); h->have_geom = false; return rc; }
    // host copies for the dose normalisation; the phantoms of the previous
    // call keep their storage, so a caller who uploads the same phantoms every
    // step reallocates nothing
    h->phantoms.resize(n);
    for (int k = 0; k < n; ++k) {
        const egsgpu_phantom &q = ph[k];
        egsgpu_handle::Phantom &P = h->phantoms[k];
        const long long nv = off[k + 1] - off[k];
        P.nx = q.nx; P.ny = q.ny; P.nz = q.nz;
        P.xb.assign(q.xb, q.xb + q.nx + 1); P.yb.assign(q.yb, q.yb + q.ny + 1); P.zb.assign(q.zb, q.zb + q.nz + 1);
        P.med.resize(nv); P.rhor.resize(nv);
        P.voff = off[k]; P.histories = q.histories; P.nhist = 0;
    }
    phantoms_parallel(off, [&](int k, long long b, long long e) {
        egsgpu_handle::Phantom &P = h->phantoms[k];
        std::copy(ph[k].med + b, ph[k].med + e, P.med.begin() + b);
        std::copy(ph[k].rhor + b, ph[k].rhor + e, P.rhor.begin() + b);
    });
    h->mvox = off[n];
    h->Smax = smax;
    h->have_geom = true;
    h->have_source = true;
    h->nhist = 0; h->nbatch = 0;
    return 0;
}

int egsgpu_run_phantoms(egsgpu_handle *h, int n_batch, void *stream) {
    if (!h || n_batch < 1) return EGSGPU_ERR_ARG;
    if (!h->multi()) { h->err = "no phantoms set"; return EGSGPU_ERR_STATE; }
    for (auto &P : h->phantoms)
        if (P.histories > 0 && P.histories < n_batch) { h->err = "a phantom has fewer histories than batches"; return EGSGPU_ERR_ARG; }
    int rc = h->eng->run_multi(h->Smax, n_batch, (cudaStream_t)stream, h->err);
    if (rc) return rc;
    for (auto &P : h->phantoms) { P.nhist += P.histories; h->nhist += P.histories; }
    h->nbatch += n_batch;
    return 0;
}

int egsgpu_get_phantom_info(egsgpu_handle *h, int k, long long *out) {
    if (!h || !out || k < 0 || k >= (int)h->phantoms.size()) return EGSGPU_ERR_ARG;
    const auto &P = h->phantoms[k];
    out[0] = P.voff; out[1] = (long long)P.nx * P.ny * P.nz; out[2] = P.nhist;
    return 0;
}

}  // extern "C"

extern "C" {

int egsgpu_get_phantom_dose(egsgpu_handle *h, int k, double *dose, double *sigma) {
    if (!h || !dose || k < 0 || k >= (int)h->phantoms.size()) return EGSGPU_ERR_ARG;
    const auto &P = h->phantoms[k];
    long long nv = (long long)P.nx * P.ny * P.nz;
    std::vector<double> s(nv), s2(nv);
    int rc = h->eng->read_sums(P.voff, nv, s.data(), s2.data(), h->err);
    if (rc) return rc;
    const double N = (double)P.nhist, nb = (double)h->nbatch;
    for (long long i = 0; i < nv; ++i) {
        int iz = (int)(i / ((long long)P.nx * P.ny)), rr = (int)(i - (long long)iz * P.nx * P.ny);
        int iy = rr / P.nx, ix = rr - iy * P.nx;
        double vol = (P.xb[ix + 1] - P.xb[ix]) * (P.yb[iy + 1] - P.yb[iy]) * (P.zb[iz + 1] - P.zb[iz]);
        double mass = vol * P.rhor[i] * h->H.media[P.med[i]].rho;
        double norm = N > 0 ? 1.602e-10 / (mass * N) : 0;   // egs_dose_scoring.cpp:318-319
        dose[i] = s[i] * norm;
        if (sigma) {
            double mean = s[i] / nb, var = nb > 1 ? (s2[i] / nb - mean * mean) / (nb - 1) : 0;
            sigma[i] = (var > 0 ? std::sqrt(var) * nb : 0) * norm;
        }
    }
    return 0;
}

int egsgpu_reset(egsgpu_handle *h) {
    if (!h || !h->have_geom) return EGSGPU_ERR_STATE;
    int rc = h->eng->clear_tallies(h->nvox(), h->err);
    if (rc) return rc;
    h->nhist = 0; h->nbatch = 0;
    for (auto &P : h->phantoms) P.nhist = 0;
    return 0;
}

int egsgpu_get_profile(egsgpu_handle *h, double *out) {
    // out[18]; see include/egsgpu.h
    if (!h || !out || !h->have_geom) return EGSGPU_ERR_ARG;
    return h->eng->read_profile(out, h->err);
}

int egsgpu_get_tallies(egsgpu_handle *h, double *sum, double *sum2, double *totals) {
    if (!h || !h->have_geom) return EGSGPU_ERR_STATE;
    return get_tallies_impl(h, sum, sum2, totals);
}

int egsgpu_get_dose(egsgpu_handle *h, double *dose, double *sigma) {
    if (!h || !h->have_geom || !dose) return EGSGPU_ERR_ARG;
    if (h->multi()) { h->err = "several phantoms are set: use egsgpu_get_phantom_dose"; return EGSGPU_ERR_STATE; }
    long long nv = h->nvox();
    std::vector<double> s(nv), s2(nv);
    int rc = egsgpu_get_tallies(h, s.data(), s2.data(), nullptr);
    if (rc) return rc;
    const double N = (double)h->nhist, nb = (double)h->nbatch;
    for (long long i = 0; i < nv; ++i) {
        int iz = (int)(i / ((long long)h->nx * h->ny)), rr = (int)(i - (long long)iz * h->nx * h->ny);
        int iy = rr / h->nx, ix = rr - iy * h->nx;
        double vol = (h->xb[ix + 1] - h->xb[ix]) * (h->yb[iy + 1] - h->yb[iy]) * (h->zb[iz + 1] - h->zb[iz]);
        double mass = vol * h->rhor[i] * h->H.media[h->med[i]].rho;
        double norm = N > 0 ? 1.602e-10 / (mass * N) : 0;   // egs_dose_scoring.cpp:318-319
        dose[i] = s[i] * norm;
        if (sigma) {
            // batch method: sigma of the mean of nb batch totals
            double mean = s[i] / nb, var = nb > 1 ? (s2[i] / nb - mean * mean) / (nb - 1) : 0;
            sigma[i] = (var > 0 ? std::sqrt(var) * nb : 0) * norm;
        }
    }
    return 0;
}

int egsgpu_adjoint(egsgpu_handle *h, long long first, long long n, uint32_t seed, const double *dL_dD,
                   double *dL_drhor) {
    if (!h || !dL_dD || !dL_drhor || n < 1 || first < 0 || first + n > 0xffffffffLL) return EGSGPU_ERR_ARG;
    if (!h->have_media || !h->have_geom || !h->have_source || h->multi()) {
        h->err = "media, one geometry and a source must be set";
        return EGSGPU_ERR_STATE;
    }
    if (h->nhist != n) { h->err = "the tallies must hold exactly the n histories being differentiated"; return EGSGPU_ERR_STATE; }
    long long nv = h->nvox();
    std::vector<double> s(nv), w(nv), D(nv);
    int rc = egsgpu_get_tallies(h, s.data(), nullptr, nullptr);
    if (rc) return rc;
    for (long long i = 0; i < nv; ++i) {
        int iz = (int)(i / ((long long)h->nx * h->ny)), rr = (int)(i - (long long)iz * h->nx * h->ny);
        int iy = rr / h->nx, ix = rr - iy * h->nx;
        double vol = (h->xb[ix + 1] - h->xb[ix]) * (h->yb[iy + 1] - h->yb[iy]) * (h->zb[iz + 1] - h->zb[iz]);
        double norm = 1.602e-10 / (vol * h->rhor[i] * h->H.media[h->med[i]].rho * (double)n);
        D[i] = s[i] * norm;
        w[i] = dL_dD[i] * norm;   // dL/dE_v
    }
    rc = h->eng->adjoint(h->S, first, n, seed, w.data(), dL_drhor, h->err);
    if (rc) return rc;
    // D = E / (rho V): the explicit dependence on the voxel's own density
    for (long long i = 0; i < nv; ++i) dL_drhor[i] -= dL_dD[i] * D[i] / h->rhor[i];
    return 0;
}

int egsgpu_set_history_tally(egsgpu_handle *h, long long first, long long n) {
    if (!h || n < 0 || n > (1LL << 24)) return EGSGPU_ERR_ARG;
    return h->eng->history_tally(first, n, h->err);
}

int egsgpu_get_history_tally(egsgpu_handle *h, double *out) {
    if (!h || !out) return EGSGPU_ERR_ARG;
    return h->eng->read_history_tally(out, h->err);
}

int egsgpu_geometry_query(egsgpu_handle *h, int op, long long n, const int32_t *ireg, const double *x,
                          const double *u, double *t, int32_t *inew) {
    if (!h) return EGSGPU_ERR_ARG;
    if (!h->have_geom) { h->err = "geometry not set"; return EGSGPU_ERR_STATE; }
    return h->eng->geometry_query(op, n, ireg, x, u, t, inew, h->err);
}

// Checkpoint layout: magic, nvox, nhist, nbatch, energy[2], counters[8], sum[nvox], sum2[nvox]
int egsgpu_checkpoint(egsgpu_handle *h, void *buf, size_t *size) {
    if (!h || !size || !h->have_geom) return EGSGPU_ERR_ARG;
    long long nv = h->nvox();
    size_t need = 8 * 4 + 2 * 8 + 8 * 8 + 2 * nv * 8;
    if (!buf) { *size = need; return 0; }
    if (*size < need) { *size = need; h->err = "checkpoint buffer too small"; return EGSGPU_ERR_ARG; }
    char *b = (char *)buf;
    long long hdr[4] = {0x45475347505531LL, nv, h->nhist, h->nbatch};
    std::memcpy(b, hdr, 32);
    double en[2];
    unsigned long long c[CNT_N];
    if (int rc = h->eng->read_totals(en, c, h->err)) return rc;
    std::memcpy(b + 32, en, 16);
    std::memcpy(b + 48, c, 64);   // the first 8 counters
    std::vector<double> s(nv), s2(nv);
    if (int rc = h->eng->read_sums(0, nv, s.data(), s2.data(), h->err)) return rc;
    std::memcpy(b + 112, s.data(), nv * 8);
    std::memcpy(b + 112 + nv * 8, s2.data(), nv * 8);
    *size = need;
    return 0;
}

int egsgpu_restore(egsgpu_handle *h, const void *buf, size_t size) {
    if (!h || !buf || !h->have_geom) return EGSGPU_ERR_ARG;
    long long nv = h->nvox();
    size_t need = 8 * 4 + 2 * 8 + 8 * 8 + 2 * nv * 8;
    const char *b = (const char *)buf;
    long long hdr[4];
    if (size < need) { h->err = "checkpoint too small"; return EGSGPU_ERR_ARG; }
    std::memcpy(hdr, b, 32);
    if (hdr[0] != 0x45475347505531LL || hdr[1] != nv) { h->err = "checkpoint does not match this geometry"; return EGSGPU_ERR_ARG; }
    double en[2];
    unsigned long long c[8];
    std::vector<double> s(nv), s2(nv);
    std::memcpy(en, b + 32, 16);
    std::memcpy(c, b + 48, 64);
    std::memcpy(s.data(), b + 112, nv * 8);
    std::memcpy(s2.data(), b + 112 + nv * 8, nv * 8);
    int rc = h->eng->restore_sums(en, c, s.data(), s2.data(), nv, h->err);
    if (rc) return rc;
    h->nhist = hdr[2];
    h->nbatch = (int)hdr[3];
    return 0;
}

// Host-only: the checkpoint of the union of two runs of the same phantom
// (the .egsdat combine of egs_application.cpp:624-660, addState): histories,
// batches, energy totals, counters and the per-voxel batch sums and sums of
// squares add.  Batch-wise uncertainties need equal histories per batch, so
// shards whose histories per batch differ are refused.
int egsgpu_combine_checkpoints(const void *a, size_t na, const void *b, size_t nb, void *out, size_t *nout) {
    if (!a || !b || !nout || na < 112 || nb < 112) return EGSGPU_ERR_ARG;
    long long ha[4], hb[4];
    std::memcpy(ha, a, 32);
    std::memcpy(hb, b, 32);
    const long long magic = 0x45475347505531LL;
    if (ha[0] != magic || hb[0] != magic || ha[1] != hb[1] || ha[1] < 0) return EGSGPU_ERR_ARG;
    const long long nv = ha[1];
    const size_t need = 8 * 4 + 2 * 8 + 8 * 8 + 2 * (size_t)nv * 8;
    if (na < need || nb < need) return EGSGPU_ERR_ARG;
    if (!out) { *nout = need; return 0; }
    if (*nout < need) { *nout = need; return EGSGPU_ERR_ARG; }
    if (ha[3] > 0 && hb[3] > 0 && ha[2] * hb[3] != hb[2] * ha[3]) return EGSGPU_ERR_ARG;
    const char *pa = (const char *)a, *pb = (const char *)b;
    char *po = (char *)out;
    long long ho[4] = {magic, nv, ha[2] + hb[2], ha[3] + hb[3]};
    std::memcpy(po, ho, 32);
    double ea[2], eb[2];
    std::memcpy(ea, pa + 32, 16);
    std::memcpy(eb, pb + 32, 16);
    ea[0] += eb[0];
    ea[1] += eb[1];
    std::memcpy(po + 32, ea, 16);
    unsigned long long ca[8], cb[8];
    std::memcpy(ca, pa + 48, 64);
    std::memcpy(cb, pb + 48, 64);
    for (int k = 0; k < 8; ++k) ca[k] += cb[k];
    std::memcpy(po + 48, ca, 64);
    for (long long i = 0; i < 2 * nv; ++i) {
        double x, y;
        std::memcpy(&x, pa + 112 + 8 * i, 8);
        std::memcpy(&y, pb + 112 + 8 * i, 8);
        x += y;
        std::memcpy(po + 112 + 8 * i, &x, 8);
    }
    *nout = need;
    return 0;
}

}  // extern "C"

// Scratch of egsgpu_run_noalloc, the entry point for callers that may not
// allocate device memory while they transport: a time-critical loop that must
// not wait on the allocator, or a host framework whose memory pool owns every
// allocation on the device.  The call still synchronises its stream once per
// wavefront round to learn whether the queues have drained.  The array
// is a fixed part of the module: it exists on every GPU the library is used
// on and costs EGSGPU_NOALLOC_SCRATCH_MIB of device memory there until the
// process exits.  Host code cannot use the name as an address; the device
// address is looked up once per device with cudaGetSymbolAddress.  All calls
// share the one array, and each call clears the counters it relies on.
static __device__ __align__(256) unsigned char g_noalloc_scratch[(size_t)EGSGPU_NOALLOC_SCRATCH_MIB << 20];
static std::mutex g_noalloc_mutex;
static unsigned char *g_noalloc_addr[256] = {};

namespace egsgpu_host {
const char *host_error();   // egs_phsp.cpp: last error of a host-only call on this thread
}

extern "C" {

int egsgpu_run_noalloc(egsgpu_handle *h, long long first, long long n, uint32_t seed, double *dose, void *stream) {
    if (!h || !dose || n < 0 || first < 0 || first + n > 0xffffffffLL) return EGSGPU_ERR_ARG;
    if (n > EGSGPU_NOALLOC_MAX_HISTORIES) {
        h->err = "egsgpu_run_noalloc: at most " + std::to_string(EGSGPU_NOALLOC_MAX_HISTORIES) +
                 " histories per call (the fixed scratch holds the particle queues of one chunk)";
        return EGSGPU_ERR_ARG;
    }
    if (!h->have_media || !h->have_geom || !h->have_source) { h->err = "media, geometry and source must be set"; return EGSGPU_ERR_STATE; }
    if (h->cfg.bca_algorithm != 0) { h->err = "egsgpu_run_noalloc uses EXACT boundary crossing only"; return EGSGPU_ERR_ARG; }
    if (h->cfg.howfarless > 0) { h->err = "egsgpu_run_noalloc transports voxel by voxel only (no HOWFARLESS)"; return EGSGPU_ERR_ARG; }
    if (h->cfg.fp64_near_faces > 0) { h->err = "egsgpu_run_noalloc runs the default FP32 step (no fp64_near_faces)"; return EGSGPU_ERR_ARG; }
    // The call synchronises its stream every round and runs as many rounds as
    // the histories need, so it cannot be recorded into a graph: refuse a
    // capturing stream before any other CUDA call, leaving the capture valid.
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    const cudaError_t ce = cudaStreamIsCapturing((cudaStream_t)stream, &cs);
    if (ce != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
        if (ce != cudaSuccess) cudaGetLastError();
        h->err = "egsgpu_run_noalloc cannot run on a capturing stream (it synchronises the stream every "
                 "wavefront round)";
        return EGSGPU_ERR_STATE;
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 256) { h->err = "no current CUDA device"; return EGSGPU_ERR_CUDA; }
    unsigned char *scratch = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_noalloc_mutex);
        if (!g_noalloc_addr[dev]) {   // first call on this device: look the array up
            void *p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess || !p) {
                h->err = std::string("cudaGetSymbolAddress(no-allocation scratch): ") + cudaGetErrorString(e);
                return EGSGPU_ERR_CUDA;
            }
            g_noalloc_addr[dev] = (unsigned char *)p;
        }
        scratch = g_noalloc_addr[dev];
    }
    if (n == 0) return 0;
    return h->eng->run_noalloc(h->S, first, n, seed, dose, (cudaStream_t)stream, scratch,
                               (size_t)EGSGPU_NOALLOC_SCRATCH_MIB << 20, h->err);
}

const char *egsgpu_last_error(egsgpu_handle *h) { return h ? h->err.c_str() : egsgpu_host::host_error(); }

void egsgpu_destroy(egsgpu_handle *h) { delete h; }

}  // extern "C"

#endif  // EGSGPU_PART_F64
