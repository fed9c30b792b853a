// ORACLE -- test infrastructure only.  Not part of the product: only tests/,
// __graft_entry__.smoke() and bench.py's CPU-baseline leg load it, as the
// checker.
//
// A scalar FP64 CPU restatement of EGSnrc's coupled photon/electron history
// loop for voxel dose (paths relative to HEN_HOUSE):
//   SHOWER / egsShower            src/egsnrc.mortran:6646-6718, interface/egs_interface2.c:92-99
//   PHOTON                        src/egsnrc.mortran:6439-6641
//   ELECTR                        src/egsnrc.mortran:985-1821
//   COMPT (bound, norej)          src/egsnrc.mortran:528-805
//   PHOTO (EADL edges)            src/egsnrc.mortran:5050-5195
//   PAIR (BH, simple angles)      src/egsnrc.mortran:4518-4715, src/egsnrc.macros:2070-2185
//   Rayleigh                      src/egsnrc.macros:1579-1613, src/egsnrc.mortran:8559-8590
//   MOLLER, BHABHA, BREMS         src/egsnrc.mortran:2599-2746, :229-307, :312-524
//   ANNIH, ANNIH_AT_REST          src/egsnrc.mortran:70-223
//   msdist_pII, mscat, sscat      src/egsnrc.mortran:4050-4294, :2984-3262
//   range / eloss / tstep macros  src/egsnrc.macros:3113-3360, :2358-2385, :1504-1512, :2491-2509
//   UPHI                          src/egsnrc.mortran:6723-6846
//   XYZ geometry                  egs++/geometry/egs_nd_geometry/egs_nd_geometry.h:769-1379
//   dose scoring                  egs++/ausgab_objects/egs_dose_scoring/egs_dose_scoring.h:203-230
//   RANMAR                        src/ranmar.mortran:67-145 (known-answer test: user_codes/ranmar_test)
// The tables come from the host data layer (egsnrc_gb300/csrc/egs_hatch.cpp),
// whose values are pinned separately against the raw data files.
//
// Pinning (the reference has no transport, dose or cross-section golden
// values, and its transport core, Mortran3 -> Fortran 77, cannot be compiled
// here without a Fortran compiler):
//   - RANMAR against the one golden vector the reference ships for this path
//     (user_codes/ranmar_test);
//   - the transport against a run of the reference itself, BEAMnrc's EXslabs
//     example: its listing and exit phase space (tests/test_oracle_exslabs.py);
//   - the XYZ geometry bit for bit, and the parallel-beam source and spectrum
//     in distribution, against the reference's own egs++ classes compiled from
//     its sources (oracle/egspp_ref.cpp, tests/test_egspp_reference.py);
//   - the interaction samplers against their cross sections: Klein-Nishina,
//     Sauter, Bethe-Heitler pair, Moller, Bhabha, bremsstrahlung, Heitler's
//     annihilation in flight, and Rayleigh with the form factors of the raw
//     pgs4form.dat (tests/test_oracle_samplers.py).
//
// Random numbers: either one RANMAR stream for the whole run (as the
// reference does) or Philox-4x32-10 (Salmon et al., SC'11) with one stream
// per particle keyed by (seed, history) and a 64-bit stream id; children get
// stream ids derived from the parent's id, draw count and child index.  The
// Philox mode consumes random numbers exactly as the GPU engine does, so the
// two can be compared history by history.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../egsnrc_gb300/csrc/egs_hatch.h"
#include "../include/egsgpu.h"

using namespace egs;

namespace {

// ------------------------------------------------------------------ RNG ----
inline void philox_round(uint32_t c[4], const uint32_t k[2]) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c[0], p1 = (uint64_t)0xCD9E8D57u * c[2];
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0, hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c[1] ^ k[0], n2 = hi0 ^ c[3] ^ k[1];
    c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
}
void philox10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c[4] = {ctr[0], ctr[1], ctr[2], ctr[3]}, k[2] = {key[0], key[1]};
    for (int r = 0; r < 10; ++r) {
        philox_round(c, k);
        k[0] += 0x9E3779B9u; k[1] += 0xBB67AE85u;
    }
    std::memcpy(out, c, 16);
}
inline uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
inline uint64_t child_sid(uint64_t sid, uint32_t n, uint32_t k) {
    return mix64(sid + 0x9E3779B97F4A7C15ull * (1 + (((uint64_t)n) << 3) + k));
}
// (x >> 9) + 0.5 scaled by 2^-23: exact in FP32 and FP64, in (0,1).
inline double u01(uint32_t x) { return ((double)(x >> 9) + 0.5) * (1.0 / 8388608.0); }

struct Ranmar {
    int u[98]; int c, cd, cm, ixx, jxx;
    int arr[128]; int seed_pos;
    void init(int ix, int jx) {   // src/ranmar.mortran:67-114
        if (ix <= 0 || ix > 31328) ix = 1802;
        if (jx <= 0 || jx > 30081) jx = 9373;
        int i = (ix / 177) % 177 + 2, j = ix % 177 + 2, k = (jx / 169) % 178 + 1, l = jx % 169;
        for (int ii = 1; ii <= 97; ++ii) {
            int s = 0, t = 8388608;
            for (int jj = 1; jj <= 24; ++jj) {
                int m = ((i * j) % 179) * k % 179;
                i = j; j = k; k = m;
                l = (53 * l + 1) % 169;
                if ((l * m) % 64 >= 32) s += t;
                t /= 2;
            }
            u[ii] = s;
        }
        c = 362436; cd = 7654321; cm = 16777213;
        ixx = 97; jxx = 33; seed_pos = 128;
    }
    void refill() {               // ranmar_get, src/ranmar.mortran:116-135
        for (int i = 0; i < 128; ++i) {
            int iopt = u[ixx] - u[jxx];
            if (iopt < 0) iopt += 16777216;
            u[ixx] = iopt;
            --ixx; --jxx;
            if (ixx == 0) ixx = 97;
            else if (jxx == 0) jxx = 97;
            c -= cd;
            if (c < 0) c += cm;
            iopt -= c;
            if (iopt < 0) iopt += 16777216;
            arr[i] = iopt;
        }
        seed_pos = 0;
    }
    double get() {
        if (seed_pos >= 128) refill();
        return arr[seed_pos++] * (1.0 / 16777216.0);
    }
};

// --------------------------------------------------------------- types ----
struct Particle {
    double E, x, y, z, u, v, w, wt;
    int iq, ir;
    uint32_t hist, n;      // history index, draws consumed
    uint64_t sid;          // stream id
    uint32_t cache[4];
    int cache_blk;
};

struct Geometry {
    int nx = 0, ny = 0, nz = 0, nxy = 0;
    std::vector<double> xb, yb, zb, rhor;
    std::vector<int> med;
    double bt = 1.0 / 4294967296.0, hbt = 0.5 / 4294967296.0;   // egs_functions.h:80-88
};

struct Source {
    egsgpu_source s{};
    std::vector<double> edges, cumw;   // histogram: alias-free inverse CDF over bins
    // alias table (egs_alias_table.cpp:117-263 layout: wi, bin)
    std::vector<double> wi;
    std::vector<int> bin;
    std::vector<float> phsp;           // phase-space particles (7 floats each)
    bool has_rot = false;              // phase-space particles rotated by s.rot
};

struct Tally {
    std::vector<double> batch, sum, sum2;
    double dep = 0, esc = 0;
    double steps = 0, psteps = 0, esteps = 0, pushes = 0;
    double tsteps = 0;   // charged-particle steps of non-zero length (AUSGAB(0) calls)
    double msdist_calls = 0;   // PRESTA-II steps (count_pII_steps, egsnrc.mortran:4163)
    // optional record of every particle that leaves the phantom, ESC_REC
    // doubles each: charge, kinetic energy, x, y, z, u, v, w, weight, history
    bool log_esc = false;
    std::vector<double> esc_log;
};
constexpr int ESC_REC = 10;

struct Oracle;

struct Run {
    Oracle *O;
    Tally *T;
    bool ranmar;
    Ranmar rm;
    uint32_t seed;
    std::vector<Particle> stack;
    double *hist_out = nullptr;
    long long hist_first = 0, hist_n = 0;
    int errors = 0;
};

struct Oracle {
    Hatch H;
    Geometry G;
    Source S;
    double ecut = 0.521, pcut = 0.01;
    std::string err;
    // HOWFARLESS (DOSXYZnrc ihowfarless = 1): transport against the outer
    // boundary only, with the floored step limits of modify_tmxs per medium
    bool hfl = false;
    std::vector<std::vector<double>> hfl_t0, hfl_t1;
};

// --------------------------------------------------------- RNG access ----
inline double rnd(Run &R, Particle &p) {
    if (R.ranmar) return R.rm.get();
    uint32_t blk = p.n >> 2;
    if ((int)blk != p.cache_blk) {
        uint32_t ctr[4] = {blk, (uint32_t)p.sid, (uint32_t)(p.sid >> 32), 0u};
        uint32_t key[2] = {R.seed, p.hist};
        philox10(ctr, key, p.cache);
        p.cache_blk = (int)blk;
    }
    return u01(p.cache[p.n++ & 3]);
}

inline void make_child(Particle &c, const Particle &parent, uint32_t k) {
    c.hist = parent.hist;
    c.sid = child_sid(parent.sid, parent.n, k);
    c.n = 0;
    c.cache_blk = -1;
}

// ------------------------------------------------------------ scoring ----
inline void score(Run &R, int ir, double edep, double wt) {
    if (ir >= 0 && edep > 0) {
        R.T->batch[ir] += edep * wt;
        R.T->dep += edep * wt;
    }
}
inline void score_hist(Run &R, const Particle &p, double e) {
    if (R.hist_out && e > 0) {
        long long i = (long long)p.hist - R.hist_first;
        if (i >= 0 && i < R.hist_n) R.hist_out[i] += e;
    }
}
inline void deposit(Run &R, const Particle &p, double edep) {
    if (p.ir >= 0 && edep > 0) {
        score(R, p.ir, edep, p.wt);
        score_hist(R, p, edep * p.wt);
    }
}
inline void escape(Run &R, const Particle &p, double e) {
    R.T->esc += e * p.wt;
    if (R.T->log_esc) {
        const double r[ESC_REC] = {(double)p.iq, p.iq == 0 ? p.E : p.E - RM, p.x, p.y, p.z, p.u, p.v, p.w, p.wt,
                                   (double)p.hist};
        R.T->esc_log.insert(R.T->esc_log.end(), r, r + ESC_REC);
    }
}

// ----------------------------------------------------------- geometry ----
int howfar(const Geometry &G, int ireg, const Particle &p, double &t) {   // egs_nd_geometry.h:963-1104
    int iz = ireg / G.nxy, ir = ireg - iz * G.nxy, iy = ir / G.nx, ix = ir - iy * G.nx;
    int inew = ireg;
    if (p.u > 0) {
        double d = (G.xb[ix + 1] - p.x) / p.u;
        if (d <= t) { t = (d <= G.bt) ? G.hbt : d; inew = (ix + 1 < G.nx) ? ireg + 1 : -1; }
    } else if (p.u < 0) {
        double d = (G.xb[ix] - p.x) / p.u;
        if (d <= t) { t = (d <= G.bt) ? G.hbt : d; inew = (ix - 1 >= 0) ? ireg - 1 : -1; }
    }
    if (p.v > 0) {
        double d = (G.yb[iy + 1] - p.y) / p.v;
        if (d <= t) { t = (d <= G.bt) ? G.hbt : d; inew = (iy + 1 < G.ny) ? ireg + G.nx : -1; }
    } else if (p.v < 0) {
        double d = (G.yb[iy] - p.y) / p.v;
        if (d <= t) { t = (d <= G.bt) ? G.hbt : d; inew = (iy - 1 >= 0) ? ireg - G.nx : -1; }
    }
    if (p.w > 0) {
        double d = (G.zb[iz + 1] - p.z) / p.w;
        if (d <= t) { t = (d <= G.bt) ? G.hbt : d; inew = (iz + 1 < G.nz) ? ireg + G.nxy : -1; }
    } else if (p.w < 0) {
        double d = (G.zb[iz] - p.z) / p.w;
        if (d <= t) { t = (d <= G.bt) ? G.hbt : d; inew = (iz - 1 >= 0) ? ireg - G.nxy : -1; }
    }
    return inew;
}

double hownear(const Geometry &G, int ireg, const Particle &p) {   // egs_nd_geometry.h:1106-1122
    int iz = ireg / G.nxy, ir = ireg - iz * G.nxy, iy = ir / G.nx, ix = ir - iy * G.nx;
    double t = std::min(p.x - G.xb[ix], G.xb[ix + 1] - p.x);
    t = std::min(t, std::min(p.y - G.yb[iy], G.yb[iy + 1] - p.y));
    t = std::min(t, std::min(p.z - G.zb[iz], G.zb[iz + 1] - p.z));
    return t;
}

// EGS_PlanesT::isWhere + EGS_BaseGeometry::findRegion (egs_planes.h:301-311,
// egs_base_geometry.h:178-190): b[hi-1] < x <= b[hi], so a point on an
// interior plane belongs to the slab below it.
int plane_where(const std::vector<double> &b, double x) {
    int n = (int)b.size() - 1;
    if (x < b[0] || x > b[n]) return -1;
    int lo = 0, hi = n;
    while (hi - lo > 1) {
        int mid = (lo + hi) / 2;
        if (x <= b[mid]) hi = mid; else lo = mid;
    }
    return hi - 1;
}

int is_where(const Geometry &G, double x, double y, double z) {
    int ix = plane_where(G.xb, x); if (ix < 0) return -1;
    int iy = plane_where(G.yb, y); if (iy < 0) return -1;
    int iz = plane_where(G.zb, z); if (iz < 0) return -1;
    return ix + iy * G.nx + iz * G.nxy;
}

// ------------------------------------------------- HOWFARLESS geometry ----
// DOSXYZnrc HOWFAR / HOWNEAR with howfarless (dosxyznrc.mortran:4177-4200,
// :4351-4355): distances to the phantom's outer faces only.
double hfl_dist_out(const Geometry &G, const Particle &p) {
    double d = 1e20;
    if (p.u > 0) d = std::min(d, (G.xb[G.nx] - p.x) / p.u); else if (p.u < 0) d = std::min(d, (G.xb[0] - p.x) / p.u);
    if (p.v > 0) d = std::min(d, (G.yb[G.ny] - p.y) / p.v); else if (p.v < 0) d = std::min(d, (G.yb[0] - p.y) / p.v);
    if (p.w > 0) d = std::min(d, (G.zb[G.nz] - p.z) / p.w); else if (p.w < 0) d = std::min(d, (G.zb[0] - p.z) / p.w);
    return d;
}
double hfl_hownear(const Geometry &G, const Particle &p) {
    double t = std::min(p.x - G.xb[0], G.xb[G.nx] - p.x);
    t = std::min(t, std::min(p.y - G.yb[0], G.yb[G.ny] - p.y));
    return std::min(t, std::min(p.z - G.zb[0], G.zb[G.nz] - p.z));
}
int hfl_howfar(const Geometry &G, const Particle &p, double &t) {
    double d = hfl_dist_out(G, p);
    if (d <= t) { t = (d <= G.bt) ? G.hbt : d; return -1; }
    return p.ir;
}
// voxel holding a point, indices clamped into the phantom
int hfl_locate(const Geometry &G, double x, double y, double z) {
    auto idx = [](const std::vector<double> &b, double v) {
        int n = (int)b.size() - 1;
        if (v <= b[0]) return 0;
        if (v >= b[n]) return n - 1;
        int lo = 0, hi = n;
        while (hi - lo > 1) { int mid = (lo + hi) / 2; if (v < b[mid]) hi = mid; else lo = mid; }
        return lo;
    };
    return idx(G.xb, x) + idx(G.yb, y) * G.nx + idx(G.zb, z) * G.nxy;
}

// HOWFARLESS dose deposition of one charged-particle step
// (dosxyznrc.mortran:3569-3760).  The step from (xi, ui) to the particle's
// end point (p.x, ...) with end direction (p.u, ...) and path length tv is
// replaced by two straight segments joined at a hinge -- placed, with equal
// probability, from the initial or from the final direction; a step without
// multiple scattering is one straight segment -- and the step's energy edep
// is shared among the voxels the segments cross in proportion to the path
// length in each.  p.ir is the voxel holding the start.  Returns the voxel
// where the segments end, or -1 when they leave the phantom; `lost` receives
// the energy beyond that point, which is not deposited.
int hfl_hinge(Run &R, Particle &p, const Geometry &G, const double xi0[3], const double ui0[3], double tv,
              bool ch_step, double edep, double &lost) {
    lost = 0;
    int loc = p.ir, iz = loc / G.nxy, rr = loc - iz * G.nxy, iy = rr / G.nx, ix = rr - iy * G.nx;
    const double pe[3] = {p.x, p.y, p.z}, ue[3] = {p.u, p.v, p.w};
    if (pe[0] > G.xb[ix] && pe[0] < G.xb[ix + 1] && pe[1] > G.yb[iy] && pe[1] < G.yb[iy + 1] &&
        pe[2] > G.zb[iz] && pe[2] < G.zb[iz + 1]) {   // the whole step stays in the voxel
        score(R, p.ir, edep, p.wt);
        score_hist(R, p, edep * p.wt);
        return p.ir;
    }
    double d[3] = {pe[0] - xi0[0], pe[1] - xi0[1], pe[2] - xi0[2]};
    double d2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    double t[2] = {tv, 0}, u[2][3] = {{ui0[0], ui0[1], ui0[2]}, {0, 0, 0}};
    if (ch_step) {
        if (rnd(R, p) < 0.5) {   // hinge from the initial direction
            double c = 1 - (d[0] * u[0][0] + d[1] * u[0][1] + d[2] * u[0][2]) / tv;
            if (c < 1e-3) {
                t[0] = std::sqrt(d2);
                for (int k = 0; k < 3; ++k) u[0][k] = d[k] / t[0];
                t[1] = 0;
            } else {
                t[0] = (tv * tv - d2) / (2 * tv * c);
                t[1] = tv - t[0];
                for (int k = 0; k < 3; ++k) u[1][k] = (d[k] - t[0] * u[0][k]) / (tv - t[0]);
            }
        } else {                 // hinge from the final direction
            for (int k = 0; k < 3; ++k) u[1][k] = ue[k];
            double c = 1 - (d[0] * u[1][0] + d[1] * u[1][1] + d[2] * u[1][2]) / tv;
            if (c < 1e-3) {
                t[0] = std::sqrt(d2);
                for (int k = 0; k < 3; ++k) u[0][k] = d[k] / t[0];
                t[1] = 0;
            } else {
                t[1] = (tv * tv - d2) / (2 * tv * c);
                t[0] = tv - t[1];
                for (int k = 0; k < 3; ++k) u[0][k] = (d[k] - t[1] * u[1][k]) / (tv - t[1]);
            }
        }
    }
    const double ttot = t[0] + t[1], frac = edep / ttot;
    const std::vector<double> *B[3] = {&G.xb, &G.yb, &G.zb};
    const int n[3] = {G.nx, G.ny, G.nz}, stride[3] = {1, G.nx, G.nxy};
    int idx[3] = {ix, iy, iz}, cur = loc;
    double pos[3] = {xi0[0], xi0[1], xi0[2]}, done = 0;
    for (int s = 0; s < 2; ++s) {
        if (!(t[s] > 0)) continue;
        if (s == 1)
            for (int k = 0; k < 3; ++k) pos[k] += u[0][k] * t[0];
        int dir[3];
        double dist[3], inv[3];
        for (int k = 0; k < 3; ++k) {
            const std::vector<double> &b = *B[k];
            if (u[s][k] > 0) { inv[k] = 1 / std::fabs(u[s][k]); dir[k] = 1; dist[k] = (b[idx[k] + 1] - pos[k]) * inv[k]; }
            else if (u[s][k] < 0) { inv[k] = 1 / std::fabs(u[s][k]); dir[k] = -1; dist[k] = (pos[k] - b[idx[k]]) * inv[k]; }
            else { inv[k] = 0; dir[k] = 0; dist[k] = 1e20; }
        }
        double walked = 0;
        while (true) {
            double dmax = t[s] - walked, dl;
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
                    dist[a] = ((*B[a])[idx[a] + 1] - (*B[a])[idx[a]]) * inv[a];
                } else out = true;
            }
            score(R, cur, dl * frac, p.wt);
            score_hist(R, p, dl * frac * p.wt);
            done += dl;
            walked += dl;
            if (out) { lost = edep - done * frac; return -1; }
            cur = next;
            if (walked >= t[s]) break;
        }
    }
    return cur;
}

// egs_nd_geometry.h:1281-1379: entry from outside; returns region, t updated.
int howfar_from_out(const Geometry &G, Particle &p, double &t) {
    const std::vector<double> *pl[3] = {&G.xb, &G.yb, &G.zb};
    double pos[3] = {p.x, p.y, p.z}, dir[3] = {p.u, p.v, p.w};
    int n[3] = {G.nx, G.ny, G.nz};
    for (int a = 0; a < 3; ++a) {
        const auto &b = *pl[a];
        int i = -1; double t1 = 0;
        if (pos[a] <= b[0] && dir[a] > 0) { t1 = (b[0] - pos[a]) / dir[a]; i = 0; }
        else if (pos[a] >= b[n[a]] && dir[a] < 0) { t1 = (b[n[a]] - pos[a]) / dir[a]; i = n[a] - 1; }
        if (i >= 0 && t1 <= t) {
            double q[3] = {pos[0] + dir[0] * t1, pos[1] + dir[1] * t1, pos[2] + dir[2] * t1};
            int idx[3];
            bool ok = true;
            for (int c = 0; c < 3; ++c) {
                if (c == a) { idx[c] = i; continue; }
                idx[c] = plane_where(*pl[c], q[c]);
                if (idx[c] < 0) { ok = false; break; }
            }
            if (ok) {
                int inew = idx[0] + idx[1] * G.nx + idx[2] * G.nxy;
                if (t1 < G.bt) {   // howfar may shorten t1 (egs_nd_geometry.h:1303-1308)
                    Particle tp = p; tp.x = q[0]; tp.y = q[1]; tp.z = q[2];
                    int itest = howfar(G, inew, tp, t1);
                    if (itest == -1 && t1 < G.bt) return -1;
                }
                t = t1;
                return inew;
            }
        }
    }
    return -1;
}

// ---------------------------------------------------------- helpers ----
struct Azim { double c, s; };
inline Azim azimuth(Run &R, Particle &p) {   // $SELECT-AZIMUTHAL-ANGLE, egsnrc.macros:2491-2509
    double xphi, xphi2, yphi, yphi2, rhophi2;
    do {
        xphi = rnd(R, p); xphi = 2 * xphi - 1; xphi2 = xphi * xphi;
        yphi = rnd(R, p); yphi2 = yphi * yphi;
        rhophi2 = xphi2 + yphi2;
    } while (rhophi2 > 1);
    rhophi2 = 1 / rhophi2;
    return {(xphi2 - yphi2) * rhophi2, 2 * xphi * yphi * rhophi2};
}
// UPHI :ADJUST: rotation of direction (a,b,c) by (sinthe,costhe,cosphi,sinphi)
inline void rotate(double a, double b, double c, double sinthe, double costhe, Azim az,
                   double &u, double &v, double &w) {
    double sinps2 = a * a + b * b;
    if (sinps2 < 1e-20) {
        u = sinthe * az.c; v = sinthe * az.s; w = c * costhe;
    } else {
        double sinpsi = std::sqrt(sinps2), us = sinthe * az.c, vs = sinthe * az.s;
        double sindel = b / sinpsi, cosdel = a / sinpsi;
        u = c * cosdel * us - sindel * vs + a * costhe;
        v = c * sindel * us + cosdel * vs + b * costhe;
        w = -sinpsi * us + c * costhe;
    }
}

inline int interval(double x, double c1, double c0) { return (int)(c1 * x + c0); }   // 1-based

// ----------------------------------------------------- photon samplers ----
struct PhotonCtx { double gle; int lgle; double cohfac; };

void rayleigh_sample(Run &R, Particle &p, const Medium &m, const PhotonCtx &pc, double &costhe,
                     double &sinthe) {   // egs_rayleigh_sampling, egsnrc.mortran:8559-8590
    const double hc_i = 80.65506856998, twice_hc2 = 0.000307444456;
    const double dwi = RAYCDFSIZE - 1;
    int l = pc.lgle - 1;
    double pmax = m.pmax1[l] * pc.gle + m.pmax0[l], xmax = hc_i * p.E, csqthe, xv;
    double rn1;
    do {
        rn1 = rnd(R, p);
        do {
            double r0 = rnd(R, p) * pmax;
            int ibin = 1 + (int)(r0 * dwi);
            int ib = m.i_array[ibin - 1];
            if (m.i_array[ibin] > ib) {
                while (!(r0 < m.fcum[ib])) ++ib;   // fcum(ib+1) 1-based
            }
            r0 = (r0 - m.fcum[ib - 1]) * m.c_array[ib - 1];
            xv = m.xgrid[ib - 1] * std::exp(std::log(1 + r0) * m.b_array[ib - 1]);
        } while (!(xv < xmax));
        xv = xv / p.E;
        costhe = 1 - twice_hc2 * xv * xv;
        csqthe = costhe * costhe;
    } while (!(2 * rn1 < 1 + csqthe));
    sinthe = std::sqrt(1.0 - csqthe);
}

// COMPT, bound Compton with resampling (ibcmp = 3), egsnrc.mortran:528-805.
// Returns the local binding-energy deposition; fills the scattered photon
// (in place) and the electron.
// With bound = false, Klein-Nishina scattering on free electrons (the
// ibcmp = 0 path of COMPT, :552-640 without the shell and pz sampling); used
// by the tests of the Klein-Nishina sampler alone.
double compton(Run &R, Particle &p, const Medium &m, Particle &el, bool bound = true) {
    const Hatch &H = R.O->H;
    double peig = p.E, ko = peig / RM, broi = 1 + 2 * ko;
    bool first_time = true;
    double Uj = 0, Jo = 0, br = 0, temp = 0, sinthe = 0, costhe = 0;
    double alph1 = 0, alph2 = 0, alpha = 0, bro = 0, broi2 = 0, bro1 = 0, rejmax = 0;
    int j = 0;
resample:
    if (bound) {
        double r17 = rnd(R, p);
        r17 = 1 + r17 * m.n_shell;
        int i = (int)r17;
        if (r17 > m.eno_array[i - 1]) i = m.eno_atbin_array[i - 1];
        j = m.shell_array[i - 1];
        Uj = H.shells.be[j];
        if (ko <= Uj) goto resample;
        Jo = H.shells.Jo[j];
    }
resample_kn:
    if (ko > 2) {
        if (first_time) {
            broi2 = broi * broi; alph1 = std::log(broi); bro = 1 / broi;
            alph2 = ko * (broi + 1) * bro * bro; alpha = alph1 + alph2;
        }
        double r15, r16, r19, aux, rejf3;
        do {
            r15 = rnd(R, p); r16 = rnd(R, p);
            if (r15 * alpha < alph1) br = std::exp(alph1 * r16) * bro;
            else br = std::sqrt(r16 * broi2 + (1 - r16)) * bro;
            temp = (1 - br) / (ko * br);
            sinthe = std::max(0., temp * (2 - temp));
            aux = 1 + br * br;
            rejf3 = aux - br * sinthe;
            r19 = rnd(R, p);
        } while (!(r19 * aux <= rejf3));
    } else {
        if (first_time) { bro = 1. / broi; bro1 = 1 - bro; rejmax = broi + bro; }
        double r15, r16, rejf3;
        do {
            r15 = rnd(R, p); r16 = rnd(R, p);
            br = bro + bro1 * r15;
            temp = (1 - br) / (ko * br);
            sinthe = std::max(0., temp * (2 - temp));
            rejf3 = 1 + br * br - br * sinthe;
        } while (!(r16 * br * rejmax <= rejf3));
    }
    first_time = false;
    if (br < bro || br > 1) goto resample_kn;
    costhe = 1 - temp;
    if (bound) {
        double br2 = br * br, aux = ko * (ko - Uj) * temp, aux1 = 2 * aux + Uj * Uj;
        double pzmax = aux - Uj;
        if (pzmax < 0 && pzmax * pzmax >= aux1) goto resample;
        pzmax = pzmax / std::sqrt(aux1);
        double qc2 = 1 + br * br - 2 * br * costhe, qc = std::sqrt(qc2);
        double af, Fmax, fpz, fpz1;
        if (pzmax > 1) { pzmax = 1; af = 0; Fmax = 1; fpz = 1; goto retry_pz; }
        {
            double aux3 = 1 + 2 * Jo * std::fabs(pzmax), aux4 = 0.5 * (1 - aux3 * aux3);
            fpz = 0.5 * std::exp(aux4);
            af = qc * (1 + br * (br - costhe) / qc2);
            if (af < 0) {
                if (pzmax > 0) fpz = 1 - fpz;
                double eta = rnd(R, p);
                if (eta > fpz) goto resample;
                af = 0; Fmax = 1;
                goto retry_pz;
            }
            if (pzmax < -0.15) { Fmax = 1 - af * 0.15; fpz1 = fpz * Fmax * Jo; }
            else if (pzmax < 0.15) {
                Fmax = 1 + af * pzmax;
                aux3 = 1 / (1 + 0.33267252734 * aux3);
                aux4 = fpz * aux3 * (0.3480242 + aux3 * (-0.0958798 + aux3 * 0.7478556)) + H.shells.erfJo[j];
                if (pzmax > 0) { fpz1 = (1 - Fmax * fpz) * Jo - 0.62665706866 * af * aux4; fpz = 1 - fpz; }
                else fpz1 = Fmax * fpz * Jo - 0.62665706866 * af * aux4;
            } else { Fmax = 1 + af * 0.15; fpz1 = (1 - Fmax * fpz) * Jo; fpz = 1 - fpz; }
            double eta = rnd(R, p);
            if (eta * Jo > fpz1) goto resample;
        }
    retry_pz:
        double pz;
        {
            double r18 = rnd(R, p) * fpz;
            if (r18 < 0.5) { r18 = std::max(1e-30, 2 * r18); pz = 0.5 * (1 - std::sqrt(1 - 2 * std::log(r18))) / Jo; }
            else { r18 = 2 * (1 - r18); pz = 0.5 * (std::sqrt(1 - 2 * std::log(r18)) - 1) / Jo; }
            if (std::fabs(pz) > 1) goto retry_pz;
            if (pz < 0.15) {
                double frej = (pz < -0.15) ? 1 - af * 0.15 : 1 + af * pz;
                double eta = rnd(R, p);
                if (eta * Fmax > frej) goto retry_pz;
            }
        }
        double pz2 = pz * pz;
        if (std::fabs(pz) < 0.01) br = br * (1 + pz * (qc + (br2 - costhe) * pz));
        else {
            double a1 = 1 - pz2 * br * costhe, a2 = 1 - pz2 * br2, a3 = qc2 - br2 * pz2 * sinthe;
            if (a3 > 1e-10) br = br / a2 * (a1 + pz * std::sqrt(a3));
        }
        Uj = Uj * RM;
    }
    double pesg = br * peig, pese = peig - pesg - Uj + RM;
    sinthe = std::sqrt(sinthe);
    Azim az = azimuth(R, p);
    double a = p.u, b = p.v, c = p.w;
    rotate(a, b, c, sinthe, costhe, az, p.u, p.v, p.w);
    p.E = pesg;
    double aux = 1 + br * br - 2 * br * costhe, ce, se;
    if (aux > 1e-8) {
        ce = (1 - br * costhe) / std::sqrt(aux);
        se = (1 - ce) * (1 + ce);
        se = (se > 0) ? -std::sqrt(se) : 0;
    } else { ce = 0; se = -1; }
    el = p;
    rotate(a, b, c, se, ce, az, el.u, el.v, el.w);
    el.E = pese;
    el.iq = -1;
    return Uj;   // deposited locally: all relaxation products are sub-threshold
}

// PHOTO with EADL edges (egsnrc.mortran:5050-5195). Converts p into the
// photo-electron; returns the locally deposited vacancy energy.
double photo(Run &R, Particle &p, const Medium &m, const PhotonCtx &pc) {
    const Hatch &H = R.O->H;
    double peig = p.E, e_vac = 0;
    bool do_relax = false;
    const ElementPhoto *el = nullptr;
    if (m.nne == 1) {
        el = &H.elements[m.elem_index[0]];
    } else {
        double aux = peig * peig, aux1 = aux * peig;
        aux = aux * std::sqrt(peig);
        double sigtot = 0, probs[64];
        for (int k = 0; k < m.nne; ++k) {
            const ElementPhoto &e = H.elements[m.elem_index[k]];
            double sigma;
            if (peig > e.edge_energies[0]) {
                sigma = (e.edge_a[0] + e.edge_b[0] / peig + e.edge_c[0] / aux + e.edge_d[0] / aux1) / peig;
            } else {
                int j;
                for (j = 1; j < e.edge_number; ++j) if (peig >= e.edge_energies[j]) break;
                if (j >= e.edge_number) j = e.edge_number - 1;
                sigma = e.edge_a[j] + pc.gle * (e.edge_b[j] + pc.gle * (e.edge_c[j] + pc.gle * e.edge_d[j]));
                sigma = std::exp(sigma);
            }
            sigma *= m.pz[k];
            sigtot += sigma;
            probs[k] = sigma;
        }
        double br = rnd(R, p) * sigtot;
        int k;
        for (k = 0; k < m.nne; ++k) { br -= probs[k]; if (br <= 0) break; }
        if (k >= m.nne) k = m.nne - 1;
        el = &H.elements[m.elem_index[k]];
    }
    double enew;
    if (peig <= el->binding[MXSHELL - 1]) {
        enew = peig + RM;
    } else {
        double br = rnd(R, p);
        int k;
        for (k = 0; k < MXINTER; ++k) {
            if (peig > el->binding[k]) {
                if (br < el->interaction_prob[k]) break;
                br = (br - el->interaction_prob[k]) / (1 - el->interaction_prob[k]);
            }
        }
        if (k > 3) enew = peig + RM;   // EADL: no vacancy below L3
        else { e_vac = el->binding[k]; enew = peig - e_vac + RM; do_relax = true; }
    }
    p.iq = -1;
    p.E = enew;
    // $SELECT-PHOTOELECTRON-DIRECTION (egsnrc.macros:1916-1955)
    if (p.E > R.O->ecut) {
        double eelec = p.E, beta = std::sqrt((eelec - RM) * (eelec + RM)) / eelec, gamma = eelec / RM;
        double alpha = 0.5 * gamma - 0.5 + 1. / gamma, ratio = beta / alpha, costhe, sinth2, xi;
        while (true) {
            double rn = rnd(R, p);
            rn = 2. * rn - 1.;
            if (ratio <= 0.2) {
                double fk = rn + 0.5 * ratio * (1. - rn) * (1. + rn);
                if (gamma < 100) costhe = (beta + fk) / (1. + beta * fk);
                else if (fk > 0) costhe = 1 - (1 - fk) * (gamma - 3) / (2 * (1 + fk) * (gamma - 1) * (gamma - 1) * (gamma - 1));
                else costhe = (beta + fk) / (1. + beta * fk);
                xi = (1 + beta * fk) * gamma * gamma;
            } else {
                xi = gamma * gamma * (1. + alpha * (std::sqrt(1. + ratio * (2. * rn + ratio)) - 1.));
                costhe = (1. - 1. / xi) / beta;
            }
            sinth2 = std::max(0., (1. - costhe) * (1. + costhe));
            double rn2 = rnd(R, p);
            if (!(rn2 > 0.5 * (1. + gamma) * sinth2 * xi / gamma)) break;
        }
        double sinthe = std::sqrt(sinth2);
        Azim az = azimuth(R, p);
        double a = p.u, b = p.v, c = p.w;
        rotate(a, b, c, sinthe, costhe, az, p.u, p.v, p.w);
    }
    return do_relax ? e_vac : 0.0;
}

// PAIR (egsnrc.mortran:4518-4715) with $SET-PAIR-ANGLE iprdst = 1.
void pair(Run &R, Particle &p, const Medium &m, Particle &second) {
    double peig = p.E, eig = peig, pese1, pese2;
    int iq1, iq2;
    if (eig <= 2.1) {
        double r30 = rnd(R, p), r34 = rnd(R, p);
        pese2 = RM + 0.5 * r30 * (peig - 2 * RM);
        pese1 = peig - pese2;
        if (r34 < 0.5) { iq1 = -1; iq2 = 1; } else { iq1 = 1; iq2 = -1; }
    } else {
        int l, l1;
        double Amax, Bmax, aux1;
        if (eig < 50.) {
            l = 4; l1 = 5;
            double delta = 4 * m.delcm / eig;
            if (delta < 1) {
                Amax = m.dl[0][l] + delta * (m.dl[1][l] + delta * m.dl[2][l]);
                Bmax = m.dl[0][l1] + delta * (m.dl[1][l1] + delta * m.dl[2][l1]);
            } else {
                double aux2 = std::log(delta + m.dl[5][l]);
                Amax = m.dl[3][l] + m.dl[4][l] * aux2;
                Bmax = m.dl[3][l1] + m.dl[4][l1] * aux2;
            }
            aux1 = 1 - RMT2 / eig;
            aux1 = aux1 * aux1;
            aux1 = aux1 * Amax / 3;
            aux1 = aux1 / (Bmax + aux1);
        } else {
            l = 6;
            Amax = m.dl[0][l]; Bmax = m.dl[0][l + 1];
            aux1 = m.bpar[1] * (1 - m.bpar[0] * RM / eig);
        }
        double del0 = eig * m.delcm, Eavail = eig - RMT2, br, Eminus, rejmax, rejf, r34;
        do {
            double r30 = rnd(R, p), r31 = rnd(R, p);
            r34 = rnd(R, p);
            int lr;
            if (r30 > aux1) { br = 0.5 * r31; rejmax = Bmax; lr = l + 1; }
            else {
                double r32 = rnd(R, p), r33 = rnd(R, p);
                br = 0.5 * (1 - std::max(r31, std::max(r32, r33)));
                rejmax = Amax; lr = l;
            }
            Eminus = br * Eavail + RM;
            double Eplus = eig - Eminus, delta = del0 / (Eminus * Eplus);
            if (delta < 1) rejf = m.dl[0][lr] + delta * (m.dl[1][lr] + delta * m.dl[2][lr]);
            else rejf = m.dl[3][lr] + m.dl[4][lr] * std::log(delta + m.dl[5][lr]);
        } while (!(r34 * rejmax <= rejf));
        pese2 = Eminus;
        pese1 = peig - pese2;
        r34 = rnd(R, p);
        if (r34 < 0.5) { iq1 = -1; iq2 = 1; } else { iq1 = 1; iq2 = -1; }
    }
    // $SET-PAIR-ANGLE, iprdst = 1
    double a = p.u, b = p.v, c = p.w;
    Azim az{0, 0};
    double ese[2] = {pese1, pese2};
    double dir[2][3];
    for (int ich = 0; ich < 2; ++ich) {
        double e = ese[ich], pse = std::sqrt(std::max(0.0, (e - RM) * (e + RM)));
        double costhe = rnd(R, p);
        costhe = 1.0 - 2.0 * costhe;
        double sinthe = RM * std::sqrt((1.0 - costhe) * (1.0 + costhe)) / (pse * costhe + e);
        costhe = (e * costhe + pse) / (pse * costhe + e);
        if (ich == 0) az = azimuth(R, p);
        else sinthe = -sinthe;
        rotate(a, b, c, sinthe, costhe, az, dir[ich][0], dir[ich][1], dir[ich][2]);
    }
    second = p;
    p.E = pese1; p.iq = iq1; p.u = dir[0][0]; p.v = dir[0][1]; p.w = dir[0][2];
    second.E = pese2; second.iq = iq2; second.u = dir[1][0]; second.v = dir[1][1]; second.w = dir[1][2];
}

// ---------------------------------------------------------- MS samplers ----
struct MsState { bool find_index = true; int i = 0, j = 0; double omega2 = 0; };

void mscat(Run &R, Particle &p, double lambda, double chia2, double q1, MsState &st, double &cost,
           double &sint) {   // egsnrc.mortran:2984-3136, spin off
    const Hatch &H = R.O->H;
    if (lambda <= 13.8) {
        double sprob = rnd(R, p), explambda = std::exp(-lambda);
        if (sprob < explambda) { cost = 1; sint = 0; return; }
        double wsum = (1 + lambda) * explambda;
        if (sprob < wsum) {
            double xi = rnd(R, p);
            xi = 2 * chia2 * xi / (1 - xi + chia2);
            cost = 1 - xi;
            sint = std::sqrt(xi * (2 - xi));
            return;
        }
        if (lambda <= 1) {
            double wprob = explambda;
            wsum = explambda;
            cost = 1; sint = 0;
            int icount = 0;
            do {
                ++icount;
                if (icount > 20) break;
                wprob = wprob * lambda / icount;
                wsum += wprob;
                double xi = rnd(R, p);
                xi = 2 * chia2 * xi / (1 - xi + chia2);
                double cosz = 1 - xi, sinz = xi * (2 - xi);
                if (sinz > 1.e-20) {
                    sinz = std::sqrt(sinz);
                    xi = rnd(R, p);
                    double phi = xi * 6.2831853;
                    cost = cost * cosz - sint * sinz * std::cos(phi);
                    sint = std::sqrt(std::max(0.0, (1 - cost) * (1 + cost)));
                }
            } while (!(wsum > sprob));
            return;
        }
    }
    if (lambda <= LAMBMAX_MS) {
        if (st.find_index) {
            double llmbda = std::log(lambda);
            double ai = llmbda * H.dllambi;
            int i = (int)ai;
            ai -= i;
            double xi = rnd(R, p);
            if (xi < ai) ++i;
            int j;
            if (q1 < QMIN_MS) j = 0;
            else if (q1 < QMAX_MS) {
                double aj = q1 * H.dqmsi;
                j = (int)aj;
                aj -= j;
                xi = rnd(R, p);
                if (xi < aj) ++j;
            } else j = MS_NQ - 1;
            if (llmbda < 2.2299)
                st.omega2 = chia2 * (lambda + 4) * (1.347006 + llmbda * (0.209364 - llmbda * (0.45525 - llmbda * (0.50142 - 0.081234 * llmbda))));
            else
                st.omega2 = chia2 * (lambda + 4) * (-2.77164 + llmbda * (2.94874 - llmbda * (0.1535754 - llmbda * 0.00552888)));
            st.i = i; st.j = j;
            st.find_index = false;
        }
        double xi = rnd(R, p);
        double ak = xi * (MS_NU - 1);
        int k = (int)ak;
        ak -= k;
        size_t base = ((size_t)st.i * MS_NQ + st.j) * MS_NU;
        if (ak > H.wms[base + k]) k = H.ims[base + k];
        double a = H.fms[base + k], u = H.ums[base + k], du = H.ums[base + k + 1] - u;
        xi = rnd(R, p);
        if (std::fabs(a) < 0.2) {
            double x1 = 0.5 * (1 - xi) * a;
            u = u + xi * du * (1 + x1 * (1 - xi * a));
        } else u = u - du / a * (1 - std::sqrt(1 + xi * a * (2 + a)));
        xi = st.omega2 * u / (1 + 0.5 * st.omega2 - u);
        if (xi > 1.99999) xi = 1.99999;
        cost = 1 - xi;
        sint = std::sqrt(xi * (2 - xi));
        return;
    }
    ++R.errors;   // lambda beyond the MS table: reported as an error
    cost = 1; sint = 0;
}

// msdist_pII (egsnrc.mortran:4050-4294), spin off.
void msdist_pII(Run &R, Particle &p, const Medium &m, double e0, double eloss, double tustep,
                double rhof, int qel, double &us, double &vs, double &ws, double &xf, double &yf,
                double &zf, double &ustep) {
    (void)qel;
    double blccc = m.blcc, xcccc = m.xcc;
    double e = e0 - 0.5 * eloss, tau = e / RM, tau2 = tau * tau, epsilon = eloss / e0, epsilonp = eloss / e;
    e = e * (1 - epsilonp * epsilonp * (6 + 10 * tau + 5 * tau2) / (24 * tau2 + 72 * tau + 48));
    double p2 = e * (e + RMT2), beta2 = p2 / (p2 + RMSQ);
    double chia2 = xcccc / (4 * p2 * blccc);
    double lambda = 0.5 * tustep * rhof * blccc / beta2;
    double temp2 = 0.166666 * (4 + tau * (6 + tau * (7 + tau * (4 + tau)))) *
                   (epsilonp / ((tau + 1) * (tau + 2))) * (epsilonp / ((tau + 1) * (tau + 2)));
    lambda = lambda * (1 - temp2);
    double etap = 1, xi_corr = 1, gamma = 1, ms_corr = 1;
    chia2 = chia2 * etap;
    lambda = lambda / (etap * (1 + chia2)) * ms_corr;
    double chilog = std::log(1 + 1 / chia2);
    double q1 = 2 * chia2 * (chilog * (1 + chia2) - 1);
    gamma = 6 * chia2 * (1 + chia2) * (chilog * (1 + 2 * chia2) - 2) / q1 * gamma;
    double xi = q1 * lambda;
    MsState st;
    double w1, sint1, w2, sint2;
    mscat(R, p, lambda, chia2, xi, st, w1, sint1);
    Azim a1 = azimuth(R, p);
    mscat(R, p, lambda, chia2, xi, st, w2, sint2);
    Azim a2 = azimuth(R, p);
    double cphi1 = a1.c, sphi1 = a1.s, cphi2 = a2.c, sphi2 = a2.s;
    double u2 = sint2 * cphi2, v2 = sint2 * sphi2, u2p = w1 * u2 + sint1 * w2;
    us = u2p * cphi1 - v2 * sphi1;
    vs = u2p * sphi1 + v2 * cphi1;
    ws = w1 * w2 - sint1 * u2;
    xi = 2 * xi * xi_corr;
    double eta = rnd(R, p);
    eta = std::sqrt(eta);
    double eta1 = 0.5 * (1 - eta);
    double delta = 0.9082483 - (0.1020621 - 0.0263747 * gamma) * xi;
    double temp1 = 2 + tau;
    double temp = (2 + tau * temp1) / ((tau + 1) * temp1);
    temp = temp - (tau + 1) / ((tau + 2) * (chilog * (1 + chia2) - 1));
    temp = temp * epsilonp;
    temp1 = 1 - temp;
    delta = delta + 0.40824829 * (epsilon * (tau + 1) / ((tau + 2) * (chilog * (1 + chia2) - 1) *
                                                         (chilog * (1 + 2 * chia2) - 2)) - 0.25 * temp * temp);
    double b = eta * delta, c = eta * (1 - delta);
    double w1v2 = w1 * v2;
    double ut = b * sint1 * cphi1 + c * (cphi1 * u2 - sphi1 * w1v2) + eta1 * us * temp1;
    double vt = b * sint1 * sphi1 + c * (sphi1 * u2 + cphi1 * w1v2) + eta1 * vs * temp1;
    double wt = eta1 * (1 + temp) + b * w1 + c * w2 + eta1 * ws * temp1;
    ustep = tustep * std::sqrt(ut * ut + vt * vt + wt * wt);
    double u0 = p.u, v0 = p.v, w0 = p.w;
    double sint02 = u0 * u0 + v0 * v0;
    if (sint02 > 1e-20) {
        double sint0 = std::sqrt(sint02), sint0i = 1 / sint0, cphi0 = sint0i * u0, sphi0 = sint0i * v0;
        u2p = w0 * us + sint0 * ws;
        ws = w0 * ws - sint0 * us;
        us = u2p * cphi0 - vs * sphi0;
        vs = u2p * sphi0 + vs * cphi0;
        u2p = w0 * ut + sint0 * wt;
        wt = w0 * wt - sint0 * ut;
        ut = u2p * cphi0 - vt * sphi0;
        vt = u2p * sphi0 + vt * cphi0;
    } else { wt = w0 * wt; ws = w0 * ws; }
    xf = p.x + tustep * ut;
    yf = p.y + tustep * vt;
    zf = p.z + tustep * wt;
}

// ------------------------------------------------------ electron tables ----
struct EMedium {
    const Medium *m;
    int qel;
    double sig(double elke, int l) const {   // l is 0-based
        return qel ? m->psig1[l] * elke + m->psig0[l] : m->esig1[l] * elke + m->esig0[l];
    }
    double dedx(double elke, int l) const {
        return qel ? m->pdedx1[l] * elke + m->pdedx0[l] : m->ededx1[l] * elke + m->ededx0[l];
    }
    double dedx1(int l) const { return qel ? m->pdedx1[l] : m->ededx1[l]; }
    double range_ep(int l) const { return qel ? m->range_ep1[l] : m->range_ep0[l]; }
};

// $COMPUTE-DRANGE (egsnrc.macros:3214-3238); lel is 1-based.
inline double drange(const EMedium &em, double e1, double e2, int lel, double el1, double el2) {
    double fedep = 1 - e2 / e1;
    double elktmp = 0.5 * (el1 + el2 + 0.25 * fedep * fedep * (1 + fedep * (1 + 0.875 * fedep)));
    double dedxmid = em.dedx(elktmp, lel - 1);
    dedxmid = 1 / dedxmid;
    double aux = em.dedx1(lel - 1) * dedxmid;
    aux = aux * (1 + 2 * aux) * (fedep / (2 - fedep)) * (fedep / (2 - fedep)) / 6;
    return fedep * e1 * dedxmid * (1 + aux);
}
// $COMPUTE-ELOSS (:3290-3312)
inline double eloss(const EMedium &em, double step, double eke, double elke, int lel, double rhof) {
    double dedxmid = em.dedx(elke, lel - 1);
    double aux = em.dedx1(lel - 1) / dedxmid;
    double de = dedxmid * step * rhof;
    double fedep = de / eke;
    return de * (1 - 0.5 * fedep * aux * (1 - 0.333333 * fedep * (aux - 1 - 0.25 * fedep * (2 - aux * (4 - aux)))));
}
// $COMPUTE-ELOSS-G (:3315-3351)
inline double eloss_g(const EMedium &em, double step, double eke, double elke, int lel, double range,
                      double rhof) {
    const Medium &m = *em.m;
    double tuss = range - em.range_ep(lel - 1) / rhof;
    if (tuss >= step) return eloss(em, step, eke, elke, lel, rhof);
    int lt = lel;
    tuss = (range - step) * rhof;
    if (tuss <= 0) return eke - m.te * 0.99;
    while (tuss < em.range_ep(lt - 1)) --lt;
    double elktmp = (lt + 1 - m.eke0) / m.eke1, eketmp = m.E_array[lt];
    tuss = (em.range_ep(lt) - tuss) / rhof;
    double de = eloss(em, tuss, eketmp, elktmp, lt, rhof);
    return de + eke - eketmp;
}

// ------------------------------------------------------------ PHOTON ----
void push(Run &R, const Particle &c) { R.stack.push_back(c); R.T->pushes += 1; }

// The energy samplers of the discrete electron and positron interactions,
// shared by the transport below and by oracle_sample_interaction (which
// checks them against their cross sections).
// MOLLER (src/egsnrc.mortran:2599-2746): the fraction br of the kinetic
// energy ekin of an electron of total energy peie given to the delta ray.
double moller_br(Run &R, Particle &p, const Medium &m, double ekin, double peie) {
    double t0 = ekin / RM, e0 = t0 + 1, extrae = peie - m.thmoll, e02 = e0 * e0;
    double g2 = t0 * t0 / e02, g3 = (2 * t0 + 1) / e02, gmax = 1 + 1.25 * g2, br, rejf4, r28;
    do {
        double r27 = rnd(R, p);
        br = m.te / (ekin - extrae * r27);
        double rr = br / (1 - br);
        r28 = rnd(R, p);
        rejf4 = 1 + g2 * br * br + rr * (rr - g3);
        r28 = gmax * r28;
    } while (!(r28 <= rejf4));
    return br;
}
// BHABHA (:229-307): the fraction br of the positron's kinetic energy ekin
// given to the electron, before PEGS's swap of the two (br >= 1/2).
double bhabha_br(Run &R, Particle &p, const Medium &m, double ekin) {
    double t0 = ekin / RM, e0 = t0 + 1.;
    double yy = 1. / (t0 + 2.), e02 = e0 * e0, beta2 = (e02 - 1.) / e02;
    double ep0 = m.te / ekin, ep0c = 1. - ep0, y2 = yy * yy, yp = 1. - 2. * yy, yp2 = yp * yp;
    double b4 = yp2 * yp, b3 = b4 + yp2, b2 = yp * (3. + y2), b1 = 2. - y2, br, rejf2, r04;
    do {
        double r03 = rnd(R, p);
        br = ep0 / (1. - ep0c * r03);
        r04 = rnd(R, p);
        rejf2 = (1.0 - beta2 * br * (b1 - br * (b2 - br * (b3 - br * b4))));
    } while (!(r04 <= rejf2));
    return br;
}
// ANNIH in flight (:70-182): the energy fraction ep of the first photon, for
// a = (positron total energy + m)/m, ep0 = 1/(a + sqrt(a (a - 2))) and
// wsamp = log((1 - ep0)/ep0).
double annih_ep(Run &R, Particle &p, double a, double ep0, double wsamp) {
    double ep, r02, rejf;
    do {
        double r01 = rnd(R, p);
        ep = ep0 * std::exp(r01 * wsamp);
        r02 = rnd(R, p);
        rejf = 1 - (ep * a - 1) * (ep * a - 1) / (ep * (a * a - 2));
    } while (!(r02 <= rejf));
    return ep;
}
// BREMS (:312-524), Bethe-Heitler with the PEGS4 screening fits: the photon
// energy esg from an electron of total energy eie2 (kinetic ekin, elke =
// log ekin) with screening-fit columns l, l1.
double brems_k(Run &R, Particle &p, const Medium &m, double eie2, double ekin, double elke, int l, int l1) {
    double peie2 = eie2, brmin = m.ap / ekin, waux = elke - m.log_ap;
    double esg, pese, ese, r07, rejf;
    do {
        double r06 = rnd(R, p);
        r07 = rnd(R, p);
        double br = brmin * std::exp(r06 * waux);
        esg = ekin * br;
        pese = peie2 - esg;
        ese = pese;
        double delta = esg / eie2 / ese * m.delcm, aux = ese / eie2, phi1, phi2;
        if (delta < 1) {
            phi1 = m.dl[0][l] + delta * (m.dl[1][l] + delta * m.dl[2][l]);
            phi2 = m.dl[0][l1] + delta * (m.dl[1][l1] + delta * m.dl[2][l1]);
        } else {
            phi1 = m.dl[3][l] + m.dl[4][l] * std::log(delta + m.dl[5][l]);
            phi2 = phi1;
        }
        rejf = (1 + aux * aux) * phi1 - 2 * aux * phi2 / 3;
    } while (!(r07 < rejf));
    return esg;
}

void photon(Run &R) {
    Oracle &O = *R.O;
    const Geometry &G = O.G;
    Particle p = R.stack.back();
    R.stack.pop_back();
    if (p.ir < 0) return;
    while (true) {   // :PNEWENERGY:
        if (p.E <= O.pcut) { deposit(R, p, p.E); return; }   // :PCUT-DISCARD:
        int medium = G.med[p.ir];
        double rhor = G.rhor[p.ir];
        const Medium &m0 = O.H.media[medium];
        PhotonCtx pc;
        pc.gle = std::log(p.E);
        double r35 = rnd(R, p);
        if (r35 == 0) r35 = 1e-30;
        double dpmfp = -std::log(r35);
        pc.cohfac = 1;
        bool interact = false;
        const Medium *mp = &m0;
        while (!interact) {   // :PNEWMEDIUM:
            const Medium &m = *mp;
            pc.lgle = interval(pc.gle, m.ge1, m.ge0);
            int l = pc.lgle - 1;
            double gmfpr0 = m.gmfp1[l] * pc.gle + m.gmfp0[l];
            while (true) {   // :PTRANS:
                double rhof = rhor, gmfp = gmfpr0 / rhof;
                pc.cohfac = m.cohe1[l] * pc.gle + m.cohe0[l];
                gmfp *= pc.cohfac;
                double tstep = gmfp * dpmfp, ustep = tstep;
                if (O.hfl) {   // one flight to the interaction or out of the phantom
                    R.T->steps += 1; R.T->psteps += 1;
                    if (hfl_dist_out(G, p) <= ustep) { escape(R, p, p.E); return; }
                    p.x += p.u * ustep; p.y += p.v * ustep; p.z += p.w * ustep;
                    p.ir = hfl_locate(G, p.x, p.y, p.z);   // the voxel that scores the interaction
                    interact = true;
                    break;
                }
                int irnew = howfar(G, p.ir, p, ustep);
                R.T->steps += 1; R.T->psteps += 1;
                p.x += p.u * ustep; p.y += p.v * ustep; p.z += p.w * ustep;
                dpmfp = std::max(0.0, dpmfp - ustep / gmfp);
                if (irnew != p.ir) {
                    p.ir = irnew;
                    if (irnew < 0) { escape(R, p, p.E); return; }   // :USER-PHOTON-DISCARD:
                    int mnew = G.med[irnew];
                    rhor = G.rhor[irnew];
                    if (mnew != medium) { medium = mnew; mp = &O.H.media[medium]; break; }
                }
                if (dpmfp <= 1e-8) { interact = true; break; }
            }
        }
        const Medium &m = *mp;
        // Rayleigh (egsnrc.macros:1602-1613)
        double r37 = rnd(R, p);
        if (r37 <= 1.0 - pc.cohfac) {
            double costhe, sinthe;
            rayleigh_sample(R, p, m, pc, costhe, sinthe);
            Azim az = azimuth(R, p);
            double a = p.u, b = p.v, c = p.w;
            rotate(a, b, c, sinthe, costhe, az, p.u, p.v, p.w);
            continue;
        }
        double r36 = rnd(R, p);
        int l = pc.lgle - 1;
        double gbr1 = m.gbr11[l] * pc.gle + m.gbr10[l];
        if (r36 <= gbr1 && p.E > RMT2) {
            Particle s;
            pair(R, p, m, s);
            make_child(s, p, 0);
            push(R, p);
            push(R, s);
            return;
        }
        double gbr2 = m.gbr21[l] * pc.gle + m.gbr20[l];
        if (r36 < gbr2) {
            Particle el;
            double edep = compton(R, p, m, el);
            make_child(el, p, 0);
            if (edep > 0) deposit(R, p, edep);
            push(R, el);
            continue;   // scattered photon goes on
        }
        double edep = photo(R, p, m, pc);
        if (edep > 0) deposit(R, p, edep);
        push(R, p);     // photon became the photo-electron, same stream
        return;
    }
}

// ------------------------------------------------------------ ELECTR ----
void annih_at_rest(Run &R, Particle &p) {   // egsnrc.mortran:186-223
    double costhe = rnd(R, p);
    costhe = 2 * costhe - 1;
    double sinthe = std::sqrt(std::max(0.0, (1 - costhe) * (1 + costhe)));
    Azim az = azimuth(R, p);
    Particle g1 = p, g2 = p;
    g1.E = RM; g1.iq = 0; g1.u = sinthe * az.c; g1.v = sinthe * az.s; g1.w = costhe;
    make_child(g2, p, 0);
    g2.E = RM; g2.iq = 0; g2.u = -g1.u; g2.v = -g1.v; g2.w = -g1.w;
    push(R, g1);
    push(R, g2);
}

void electr(Run &R) {
    Oracle &O = *R.O;
    const Geometry &G = O.G;
    const TransportParams &P = O.H.params;
    Particle p = R.stack.back();
    R.stack.pop_back();
    if (p.ir < 0) return;
    int medium = G.med[p.ir];
    double rhor = G.rhor[p.ir];
newelectron:
    {
        int lelec = p.iq, qel = (1 + lelec) / 2;
        double peie = p.E, eie = peie;
        const Medium *mp = &O.H.media[medium];
        EMedium em{mp, qel};
        double eke = 0, elke = 0, sig0 = 0, demfp = 0, total_de = 0, total_tstep = 0, de = 0, range = 0;
        int lelke = 0;
        bool compute_tstep;
        if (eie <= O.ecut) goto ecut_discard;
    tstep_loop:
        compute_tstep = true;
        eke = eie - RM;
        {
            double r = rnd(R, p);
            if (r == 0) r = 1e-30;
            demfp = std::max(-std::log(r), 1e-8);
        }
        elke = std::log(eke);
        lelke = interval(elke, mp->eke1, mp->eke0);
        if (mp->sig_ismonotone[qel]) sig0 = em.sig(elke, lelke - 1) / em.dedx(elke, lelke - 1);
        else sig0 = qel ? mp->psig_e : mp->esig_e;
        while (true) {   // :USTEP:
            const Medium &m = *mp;
            double rhof = rhor, sig = sig0, tstep;
            if (sig <= 0) { tstep = 1e8; sig0 = 1e-15; }
            else {
                if (compute_tstep) {
                    total_de = demfp / sig;
                    double ekef = eke - total_de;
                    if (ekef <= m.E_array[0]) tstep = 1e8;
                    else {
                        double elkef = std::log(ekef);
                        int lelkef = interval(elkef, m.eke1, m.eke0);
                        if (lelkef == lelke) tstep = drange(em, eke, ekef, lelke, elke, elkef);
                        else {
                            double ekei = m.E_array[lelke - 1], elkei = (lelke - m.eke0) / m.eke1;
                            double tuss = drange(em, eke, ekei, lelke, elke, elkei);
                            ekei = m.E_array[lelkef];
                            elkei = (lelkef + 1 - m.eke0) / m.eke1;
                            tstep = drange(em, ekei, ekef, lelkef, elkei, elkef);
                            tstep = tstep + tuss + em.range_ep(lelke - 1) - em.range_ep(lelkef);
                        }
                    }
                    total_tstep = tstep;
                    compute_tstep = false;
                }
                tstep = total_tstep / rhof;
            }
            double dedx0 = em.dedx(elke, lelke - 1), dedx = rhof * dedx0;
            double tmxs = O.hfl ? (O.hfl_t1[medium][lelke - 1] * elke + O.hfl_t0[medium][lelke - 1]) / rhof
                                : (m.tmxs1[lelke - 1] * elke + m.tmxs0[lelke - 1]) / rhof;
            {
                double ekei = m.E_array[lelke - 1], elkei = (lelke - m.eke0) / m.eke1;
                range = drange(em, eke, ekei, lelke, elke, elkei);
                range = (range + em.range_ep(lelke - 1)) / rhof;
            }
            tmxs = std::min(tmxs, P.smaxir);
            double tustep = std::min(tstep, std::min(tmxs, range));
            double tperp = O.hfl ? hfl_hownear(G, p) : hownear(G, p.ir, p);
            double blccl = rhof * m.blcc;
            double p2 = eke * (eke + RMT2), beta2 = p2 / (p2 + RMSQ);
            double ssmfp = beta2 / blccl, skindepth = P.skindepth_for_bca * ssmfp;
            tustep = std::min(tustep, std::max(tperp, skindepth));
            bool callhowfar, dosingle = false, callmsdist, domultiple = false;
            double ustep, uscat = 0, vscat = 0, wscat = 0, xtrans = 0, ytrans = 0, ztrans = 0;
            // PRESTA-I multiple scattering of the step ($CALCULATE-XI, egsnrc.macros:1323-1348)
            double ms_beta2 = 0, ms_chia2 = 0, ms_xi = 0;
            const double xccl = rhof * m.xcc;
            auto calculate_xi = [&](double ekems, double len) {
                double pp2 = ekems * (ekems + RMT2);
                ms_beta2 = pp2 / (pp2 + RMSQ);
                ms_chia2 = xccl / (4 * blccl * pp2);
                ms_xi = 0.5 * xccl / pp2 / ms_beta2 * len;
                ms_xi = ms_xi * (std::log(1 + 1. / ms_chia2) - 1 / (1 + ms_chia2));
            };
            R.T->steps += 1; R.T->esteps += 1;
            if (tustep <= tperp && (!P.exact_bca || tustep > skindepth)) {
                callhowfar = false; callmsdist = true;
                R.T->msdist_calls += 1;
                de = eloss_g(em, tustep, eke, elke, lelke, range, rhof);
                msdist_pII(R, p, m, eke, de, tustep, rhof, qel, uscat, vscat, wscat, xtrans, ytrans, ztrans, ustep);
            } else if (P.exact_bca) {
                callmsdist = false;
                double rnnoss = rnd(R, p);
                if (rnnoss < 1.e-30) rnnoss = 1.e-30;
                double lambda = -std::log(1 - rnnoss);
                double lambda_max = 0.5 * blccl * RM / dedx * std::pow(eke / RM + 1, 3);
                if (lambda >= 0 && lambda_max > 0) {
                    double tuss = (lambda < lambda_max) ? lambda * ssmfp * (1 - 0.5 * lambda / lambda_max)
                                                         : 0.5 * lambda * ssmfp;
                    if (tuss < tustep) { tustep = tuss; dosingle = true; }
                    else dosingle = false;
                } else {
                    ++R.errors;
                    return;
                }
                ustep = tustep;
                callhowfar = !(ustep < tperp);
            } else {
                // boundary crossing a la EGS4/PRESTA-I with the exact path-length
                // correction: $SET-USTEP (egsnrc.macros:1308-1321), egsnrc.mortran:1329-1345
                callmsdist = false;
                domultiple = true;
                calculate_xi(eke - 0.5 * tustep * dedx, tustep);
                ustep = ms_xi < 0.1 ? tustep * (1 - ms_xi * (0.5 - ms_xi * 0.166667))
                                    : tustep * (1 - std::exp(-ms_xi)) / ms_xi;
                callhowfar = !(ustep < tperp);
            }
            const double ustep0 = ustep;
            int irold = p.ir, irnew = p.ir;
            if (callhowfar) irnew = O.hfl ? hfl_howfar(G, p, ustep) : howfar(G, p.ir, p, ustep);
            if (ustep <= 0) ustep = 0;
            if (ustep == 0) {
                if (irnew != irold) {
                    p.ir = irnew;
                    if (irnew < 0) { escape(R, p, (lelec < 0) ? p.E - RM : p.E + RM); return; }
                    int mnew = G.med[irnew];
                    rhor = G.rhor[irnew];
                    medium = mnew;
                    mp = &O.H.media[medium];
                    em.m = mp;
                }
                if (eie <= O.ecut) goto ecut_discard;
                goto tstep_loop;
            }
            R.T->tsteps += 1;
            double vstep = ustep, tvstep;
            if (callhowfar) {
                if (P.exact_bca) {
                    tvstep = vstep;
                    if (tvstep != tustep) dosingle = false;
                } else if (vstep < ustep0) {
                    // $SET-TVSTEP (egsnrc.macros:1350-1392)
                    calculate_xi(eke - 0.5 * tustep * vstep / ustep0 * dedx, vstep);
                    if (ms_xi < 0.1) tvstep = vstep * (1 + ms_xi * (0.5 + ms_xi * 0.333333));
                    else if (ms_xi < 0.999999) tvstep = -vstep * std::log(1 - ms_xi) / ms_xi;
                    else { ++R.errors; return; }
                } else tvstep = tustep;
                de = eloss_g(em, tvstep, eke, elke, lelke, range, rhof);
            } else {
                tvstep = tustep;
                if (!callmsdist) de = eloss_g(em, tvstep, eke, elke, lelke, range, rhof);
            }
            double save_de = de, edep = de, ekef = eke - de;
            double costhe = 1, sinthe = 0;
            if (!callmsdist && domultiple) {
                // approximate CH step: one multiple-scattering deflection (egsnrc.mortran:1480-1496)
                double lambda = blccl * tvstep / ms_beta2 / (1 + ms_chia2);
                MsState st;
                mscat(R, p, lambda, ms_chia2, ms_xi, st, costhe, sinthe);
            }
            if (!callmsdist && dosingle) {
                double ekems = std::max(ekef, O.ecut - RM);
                double pp2 = ekems * (ekems + RMT2);
                double chia2 = m.xcc / (4 * m.blcc * pp2);
                double xi = rnd(R, p);   // sscat (:3226-3262)
                xi = 2 * chia2 * xi / (1 - xi + chia2);
                costhe = 1 - xi;
                sinthe = std::sqrt(xi * (2 - xi));
            }
            double xf, yf, zf, uf, vf, wf;
            if (callmsdist) { uf = uscat; vf = vscat; wf = wscat; xf = xtrans; yf = ytrans; zf = ztrans; }
            else {
                xf = p.x + p.u * vstep; yf = p.y + p.v * vstep; zf = p.z + p.w * vstep;
                if (dosingle || domultiple) {
                    Azim az = azimuth(R, p);
                    rotate(p.u, p.v, p.w, sinthe, costhe, az, uf, vf, wf);
                } else { uf = p.u; vf = p.v; wf = p.w; }
            }
            if (O.hfl) {
                const double xi0[3] = {p.x, p.y, p.z}, ui0[3] = {p.u, p.v, p.w};
                p.x = xf; p.y = yf; p.z = zf; p.u = uf; p.v = vf; p.w = wf;
                double lost;
                int iend = hfl_hinge(R, p, G, xi0, ui0, tvstep, callmsdist, edep, lost);
                if (iend < 0) {   // the straight segments left the phantom: the particle is gone
                    double e = peie - edep;
                    escape(R, p, lost + ((lelec < 0) ? e - RM : e + RM));
                    return;
                }
                if (irnew >= 0) { p.ir = iend; irold = irnew = iend; }
            } else {
                deposit(R, p, edep);   // AUSGAB(0) in the region before transport
                p.x = xf; p.y = yf; p.z = zf; p.u = uf; p.v = vf; p.w = wf;
            }
            peie = peie - edep;
            eie = peie;
            p.E = peie;
            if (irnew == p.ir && eie <= O.ecut) goto ecut_discard;
            int medold = medium;
            eke = eie - RM;
            elke = std::log(eke);
            lelke = interval(elke, mp->eke1, mp->eke0);
            if (irnew != irold) {
                p.ir = irnew;
                if (irnew < 0) {
                    if (eie <= O.ecut) { escape(R, p, (lelec < 0) ? p.E - RM : p.E + RM); return; }
                    escape(R, p, (lelec < 0) ? p.E - RM : p.E + RM);
                    return;
                }
                medium = G.med[irnew];
                rhor = G.rhor[irnew];
                mp = &O.H.media[medium];
                em.m = mp;
            }
            if (eie <= O.ecut) goto ecut_discard;
            if (medium != medold) goto tstep_loop;
            demfp = demfp - save_de * sig;
            total_de = total_de - save_de;
            total_tstep = total_tstep - tvstep * rhof;
            if (total_tstep < 1e-9) demfp = 0;
            if (demfp < 1e-8) break;
        }
        {
            double sigf = em.sig(elke, lelke - 1) / em.dedx(elke, lelke - 1);
            double sigratio = sigf / sig0;
            double rfict = rnd(R, p);
            if (!(rfict <= sigratio)) goto tstep_loop;
        }
        // discrete interaction
        {
        const Medium &m = *mp;
        if (lelec < 0) {
            double ebr1 = m.ebr11[lelke - 1] * elke + m.ebr10[lelke - 1];
            double r24 = rnd(R, p);
            bool brems = r24 <= ebr1;
            if (!brems) {
                if (p.E <= m.thmoll) {
                    if (ebr1 <= 0) goto newelectron;
                    brems = true;
                }
            }
            if (!brems) {
                // MOLLER (:2599-2746)
                double peie2 = p.E, pekin = peie2 - RM, ekin = pekin;
                if (ekin <= 2 * m.te) goto newelectron;
                double br = moller_br(R, p, m, ekin, peie2);
                double pekse2 = br * ekin, pese1 = peie2 - pekse2, pese2 = pekse2 + RM;
                double h1 = (peie2 + RM) / pekin;
                double dcosth = h1 * (pese1 - RM) / (pese1 + RM);
                double sinthe = std::sqrt(std::max(0.0, 1 - dcosth)), costhe = std::sqrt(std::min(1.0, dcosth));
                Azim az = azimuth(R, p);
                double a = p.u, b = p.v, c = p.w;
                rotate(a, b, c, sinthe, costhe, az, p.u, p.v, p.w);
                p.E = pese1;
                Particle d = p;
                make_child(d, p, 0);
                dcosth = h1 * (pese2 - RM) / (pese2 + RM);
                sinthe = -std::sqrt(std::max(0.0, 1 - dcosth));
                costhe = std::sqrt(std::min(1.0, dcosth));
                rotate(a, b, c, sinthe, costhe, az, d.u, d.v, d.w);
                d.E = pese2; d.iq = -1;
                push(R, d);
                goto newelectron;
            }
        } else {
            double pbr1 = m.pbr11[lelke - 1] * elke + m.pbr10[lelke - 1];
            double r25 = rnd(R, p);
            if (!(r25 < pbr1)) {
                double pbr2 = m.pbr21[lelke - 1] * elke + m.pbr20[lelke - 1];
                if (r25 < pbr2) {
                    // BHABHA (:229-307)
                    double peip = p.E, pekin = peip - RM, ekin = pekin;
                    double br = bhabha_br(R, p, m, ekin);
                    int iq_np = 1, iq_new = -1;
                    if (!(br < 0.5)) { iq_np = -1; iq_new = 1; br = 1. - br; }
                    br = std::max(br, 0.0);
                    double pekse2 = br * ekin, pese1 = peip - pekse2, pese2 = pekse2 + RM;
                    double h1 = (peip + RM) / pekin;
                    double dcosth = std::min(1.0, h1 * (pese1 - RM) / (pese1 + RM));
                    double sinthe = std::sqrt(std::max(0.0, 1. - dcosth)), costhe = std::sqrt(dcosth);
                    Azim az = azimuth(R, p);
                    double a = p.u, b = p.v, c = p.w;
                    rotate(a, b, c, sinthe, costhe, az, p.u, p.v, p.w);
                    p.E = pese1; p.iq = iq_np;
                    Particle d = p;
                    make_child(d, p, 0);
                    dcosth = h1 * (pese2 - RM) / (pese2 + RM);
                    sinthe = -std::sqrt(std::max(0.0, 1. - dcosth));
                    costhe = std::sqrt(std::min(1.0, dcosth));
                    rotate(a, b, c, sinthe, costhe, az, d.u, d.v, d.w);
                    d.E = pese2; d.iq = iq_new;
                    push(R, d);
                    push(R, p);
                    return;   // both re-enter through the stack
                }
                // ANNIH in flight (:70-182)
                double pavip = p.E + RM, avip = pavip, a = avip / RM, g = a - 1.0, t = g - 1.0;
                double pp = std::sqrt(a * t), pot = pp / t, ep0 = 1.0 / (a + pp), wsamp = std::log((1.0 - ep0) / ep0);
                double aa = p.u, bb = p.v, cc = p.w;
                const double ep = annih_ep(R, p, a, ep0, wsamp);
                double esg1 = avip * ep;
                Particle g1 = p;
                g1.E = esg1; g1.iq = 0;
                double costhe = std::max(-1.0, std::min(1.0, (esg1 - RM) * pot / esg1));
                double sinthe = std::sqrt(1.0 - costhe * costhe);
                Azim az = azimuth(R, p);
                g1.n = p.n; g1.cache_blk = p.cache_blk; std::memcpy(g1.cache, p.cache, 16);
                rotate(aa, bb, cc, sinthe, costhe, az, g1.u, g1.v, g1.w);
                Particle g2 = g1;
                make_child(g2, p, 0);
                double esg2 = pavip - esg1;
                g2.E = esg2;
                costhe = std::max(-1.0, std::min(1.0, (esg2 - RM) * pot / esg2));
                sinthe = -std::sqrt(1.0 - costhe * costhe);
                rotate(aa, bb, cc, sinthe, costhe, az, g2.u, g2.v, g2.w);
                push(R, g1);
                push(R, g2);
                return;
            }
        }
        // BREMS (:312-524), BH cross section, KM angle
        {
            double peie2 = p.E, eie2 = peie2, ekin = peie2 - RM;
            int l = (eie2 < 50.0) ? 0 : 2, l1 = l + 1;
            double a = p.u, b = p.v, c = p.w, sinpsi = a * a + b * b, sindel = 0, cosdel = 0;
            if (sinpsi > 1e-20) { sinpsi = std::sqrt(sinpsi); sindel = b / sinpsi; cosdel = a / sinpsi; }
            double ztarg = m.zbrang, tteie = eie2 / RM;
            double beta = std::sqrt((tteie - 1) * (tteie + 1)) / tteie;
            double y2max = 2 * beta * (1 + beta) * tteie * tteie, y2maxi = 1 / y2max;
            double z2max = y2max + 1, z2maxi = std::sqrt(z2max);
            const double esg = brems_k(R, p, m, eie2, ekin, elke, l, l1);
            const double pese = peie2 - esg, ese = pese;
            double ttese = ese / RM, esedei = ttese / tteie, rjarg1 = 1 + esedei * esedei, rjarg2 = rjarg1 + 2 * esedei;
            double aux = 2 * ese * tteie / esg;
            aux = aux * aux;
            double aux1 = aux * ztarg, rjarg3;
            if (aux1 > 10) rjarg3 = m.lzbrang + (1 - aux1) / (aux1 * aux1);
            else rjarg3 = std::log(aux / (1 + aux1));
            double rejmax = rjarg1 * rjarg3 - rjarg2, y2tst, rtest, rejtst;
            while (true) {
                y2tst = rnd(R, p);
                rtest = rnd(R, p);
                double aux3 = z2maxi / (y2tst + (1 - y2tst) * z2maxi);
                rtest = rtest * aux3 * rejmax;
                y2tst = aux3 * aux3 - 1;
                double a34 = aux3 * aux3 * aux3 * aux3;
                double y2tst1 = esedei * y2tst / a34;
                double aux4 = 16 * y2tst1 - rjarg2, aux5 = rjarg1 - 4 * y2tst1;
                if (rtest < aux4 + aux5 * rjarg3) break;
                double aux2 = std::log(aux / (1 + aux1 / a34));
                rejtst = aux4 + aux5 * aux2;
                if (rtest < rejtst) break;
            }
            double costhe = 1 - 2 * y2tst * y2maxi;
            double sinthe = std::sqrt(std::max((1 - costhe) * (1 + costhe), 0.0));
            Azim az = azimuth(R, p);
            Particle g = p;
            make_child(g, p, 0);
            g.E = esg; g.iq = 0;
            if (sinpsi >= 1e-10) {
                double us = sinthe * az.c, vs = sinthe * az.s;
                g.u = c * cosdel * us - sindel * vs + a * costhe;
                g.v = c * sindel * us + cosdel * vs + b * costhe;
                g.w = c * costhe - sinpsi * us;
            } else { g.u = sinthe * az.c; g.v = sinthe * az.s; g.w = c * costhe; }
            push(R, g);
            p.E = pese;
            goto newelectron;
        }
        }
    ecut_discard:
        {
            double edep = p.E - RM;
            deposit(R, p, edep);
            if (lelec > 0) annih_at_rest(R, p);
            return;
        }
    }
}

// ------------------------------------------------------------- source ----
void build_alias(Source &S) {   // egs_alias_table.cpp:117-263, histogram type
    int np = S.s.nbins;
    std::vector<double> fcum(np);
    double sum = 0;
    for (int i = 0; i < np; ++i) { fcum[i] = S.s.weights[i] * (S.s.edges[i + 1] - S.s.edges[i]); sum += fcum[i]; }
    S.wi.assign(np, 1.0);
    S.bin.assign(np, 0);
    std::vector<bool> not_done(np, true);
    for (int i = 0; i < np; ++i) fcum[i] /= sum;
    // Walker alias construction
    std::vector<double> w(np);
    for (int i = 0; i < np; ++i) w[i] = fcum[i] * np;
    std::vector<int> small, large;
    for (int i = 0; i < np; ++i) (w[i] < 1 ? small : large).push_back(i);
    while (!small.empty() && !large.empty()) {
        int s = small.back(); small.pop_back();
        int lg = large.back();
        S.wi[s] = w[s];
        S.bin[s] = lg;
        w[lg] -= 1 - w[s];
        if (w[lg] < 1) { large.pop_back(); small.push_back(lg); }
    }
    for (int i : small) { S.wi[i] = 1; S.bin[i] = i; }
    for (int i : large) { S.wi[i] = 1; S.bin[i] = i; }
    S.edges.assign(S.s.edges, S.s.edges + np + 1);
}

bool source_particle(Run &R, uint32_t hist, Particle &p) {
    const Source &S = R.O->S;
    p = Particle();
    p.hist = hist; p.sid = 0; p.n = 0; p.cache_blk = -1; p.wt = 1;
    double x = S.s.pos[0], y = S.s.pos[1], z = S.s.pos[2];
    double u = S.s.dir[0], v = S.s.dir[1], w = S.s.dir[2];
    int charge = S.s.charge;
    if (S.s.shape == 1) {
        x = S.s.xmin + (S.s.xmax - S.s.xmin) * rnd(R, p);
        y = S.s.ymin + (S.s.ymax - S.s.ymin) * rnd(R, p);
    }
    double ek;
    if (S.s.shape == 2) {
        // EGS_PhspSource::getNextParticle (egs++/sources/egs_phsp_source/egs_phsp_source.cpp:284-323):
        // position in the source plane, w from u and v with the sign of the
        // weight; each particle used recycle + 1 times with its weight shared
        const float *q = S.phsp.data() + 7 * (((long long)hist / (S.s.recycle + 1)) % S.s.nphsp);
        charge = (int)q[0];
        ek = q[1];
        x += q[2]; y += q[3];
        u = q[4]; v = q[5];
        double a = u * u + v * v;
        w = a < 1 ? std::sqrt(1 - a) : 0.0;
        if (q[6] < 0) w = -w;
        p.wt = std::fabs((double)q[6]) / (S.s.recycle + 1);
        if (S.has_rot) {
            // EGS_TransformedSource (egs++/sources/egs_transformed_source) with
            // EGS_AffineTransform (egs++/egs_transformations.h:480-540):
            // position R (x, y, 0) + t, direction R u
            const double *Rm = S.s.rot, px = q[2], py = q[3], u0 = u, v0 = v, w0 = w;
            x = S.s.pos[0] + (Rm[0] * px + Rm[1] * py);
            y = S.s.pos[1] + (Rm[3] * px + Rm[4] * py);
            z = S.s.pos[2] + (Rm[6] * px + Rm[7] * py);
            u = Rm[0] * u0 + Rm[1] * v0 + Rm[2] * w0;
            v = Rm[3] * u0 + Rm[4] * v0 + Rm[5] * w0;
            w = Rm[6] * u0 + Rm[7] * v0 + Rm[8] * w0;
        }
    } else if (S.s.spectrum == 0) ek = S.s.energy;
    else {
        int np = S.s.nbins;
        double aj = rnd(R, p) * np;
        int j = (int)aj;
        aj -= j;
        if (aj > S.wi[j]) j = S.bin[j];
        ek = S.edges[j] + (S.edges[j + 1] - S.edges[j]) * rnd(R, p);
    }
    p.iq = charge;
    p.E = (p.iq == 0) ? ek : ek + RM;
    p.x = x; p.y = y; p.z = z;
    p.u = u; p.v = v; p.w = w;
    // EGS_Application::simulateSingleShower (egs_application.cpp:938-945)
    int ir = is_where(R.O->G, x, y, z);
    if (ir < 0) {
        double t = 1e30;   // veryFar, egs_functions.h:105
        ir = howfar_from_out(R.O->G, p, t);
        if (ir >= 0) { p.x += p.u * t; p.y += p.v * t; p.z += p.w * t; }
    }
    p.ir = ir;
    return ir >= 0;
}

void run_range(Oracle *O, Tally *T, long long first, long long n, int nbatch_local_dummy, uint32_t seed,
               int use_ranmar, int ranmar_ix, int ranmar_jx, double *hist_out, long long hist_first,
               long long hist_n, std::atomic<int> *errs) {
    (void)nbatch_local_dummy;
    Run R;
    R.O = O; R.T = T; R.ranmar = use_ranmar != 0; R.seed = seed;
    R.hist_out = hist_out; R.hist_first = hist_first; R.hist_n = hist_n;
    if (R.ranmar) R.rm.init(ranmar_ix, ranmar_jx);
    R.stack.reserve(4096);
    for (long long h = first; h < first + n; ++h) {
        Particle p;
        if (!source_particle(R, (uint32_t)h, p)) continue;
        R.stack.push_back(p);
        while (!R.stack.empty()) {
            if (R.stack.back().iq == 0) photon(R);
            else electr(R);
        }
    }
    if (R.errors) errs->fetch_add(R.errors);
}

}  // namespace

// ------------------------------------------------------------- C ABI ----
extern "C" {

struct oracle_handle {
    Oracle O;
    Tally T;
    long long nhist = 0;
    int nbatch = 0;
    std::vector<double> hist_buf;
    long long hist_first = 0, hist_n = 0;
};

// bca_algorithm: 0 EXACT, 1 PRESTA-I (egsnrc.mortran:2782-2783); skindepth
// in elastic MFPs (PRESTA-I with skindepth <= 1e-4: the old PRESTA default).
oracle_handle *oracle_create_bca(const char *data_dir, const char *pegs, const char *const *names, int n,
                                 double ecut, double pcut, int bca_algorithm, double skindepth) {
    auto *h = new oracle_handle();
    TransportParams tp;
    tp.ecut = ecut; tp.pcut = pcut;
    tp.exact_bca = bca_algorithm == 0;
    tp.skindepth_for_bca = skindepth;
    std::vector<std::string> nm(names, names + n);
    std::string err;
    if (hatch(data_dir, pegs, nm, tp, h->O.H, err)) {
        std::fprintf(stderr, "oracle: %s\n", err.c_str());
        delete h;
        return nullptr;
    }
    double ecut_eff = ecut, pcut_eff = pcut;
    for (auto &m : h->O.H.media) { ecut_eff = std::max(ecut_eff, m.ae); pcut_eff = std::max(pcut_eff, m.ap); }
    h->O.ecut = ecut_eff;
    h->O.pcut = pcut_eff;
    return h;
}

oracle_handle *oracle_create(const char *data_dir, const char *pegs, const char *const *names, int n,
                             double ecut, double pcut) {
    return oracle_create_bca(data_dir, pegs, names, n, ecut, pcut, 0, 3.0);
}

// The skin depth for boundary crossing in use (elastic MFPs).
double oracle_skindepth(oracle_handle *h) { return h->O.H.params.skindepth_for_bca; }
// Charged-particle steps of non-zero length so far (the AUSGAB(0) calls of
// ELECTR; BEAMnrc's "total # charged particle steps").
double oracle_charged_steps(oracle_handle *h) { return h->T.tsteps; }
// PRESTA-II (msdist) steps so far.
double oracle_msdist_steps(oracle_handle *h) { return h->T.msdist_calls; }

void oracle_destroy(oracle_handle *h) { delete h; }

int oracle_set_geometry(oracle_handle *h, int nx, int ny, int nz, const double *xb, const double *yb,
                        const double *zb, const int32_t *med, const double *rhor) {
    Geometry &G = h->O.G;
    G.nx = nx; G.ny = ny; G.nz = nz; G.nxy = nx * ny;
    G.xb.assign(xb, xb + nx + 1); G.yb.assign(yb, yb + ny + 1); G.zb.assign(zb, zb + nz + 1);
    size_t nv = (size_t)nx * ny * nz;
    G.med.assign(med, med + nv);
    G.rhor.assign(rhor, rhor + nv);
    for (size_t i = 0; i < nv; ++i)
        if (G.med[i] < 0 || G.med[i] >= (int)h->O.H.media.size()) return 1;
    h->T.batch.assign(nv, 0); h->T.sum.assign(nv, 0); h->T.sum2.assign(nv, 0);
    return 0;
}

// Geometry queries on the current phantom, as egsgpu_geometry_query: op 0
// isWhere, op 1 howfar (howfarFromOut for ireg < 0), op 2 hownear.
int oracle_geometry_query(oracle_handle *h, int op, long long n, const int32_t *ireg, const double *x,
                          const double *u, double *t, int32_t *inew) {
    const Geometry &G = h->O.G;
    const long long nv = (long long)G.nxy * G.nz;
    for (long long i = 0; i < n; ++i) {
        Particle p;
        p.x = x[3 * i]; p.y = x[3 * i + 1]; p.z = x[3 * i + 2];
        if (op == 0) {
            inew[i] = is_where(G, p.x, p.y, p.z);
        } else if (op == 1) {
            p.u = u[3 * i]; p.v = u[3 * i + 1]; p.w = u[3 * i + 2];
            if (ireg[i] >= nv) return 1;
            inew[i] = ireg[i] >= 0 ? howfar(G, ireg[i], p, t[i]) : howfar_from_out(G, p, t[i]);
        } else if (op == 2) {
            if (ireg[i] < 0 || ireg[i] >= nv) return 1;
            t[i] = hownear(G, ireg[i], p);
        } else {
            return 1;
        }
    }
    return 0;
}

// Interaction samplers alone, for the distribution tests: n interactions of
// a photon (or, for kind 2, a photo-electron) of energy E in medium `med`,
// on history streams first, first+1, ...:
//   kind 0  Klein-Nishina on free electrons: out = {k'/k, cos theta of the photon}
//   kind 1  bound Compton (ibcmp = 3):        out = {k'/k, cos theta, binding energy}
//   kind 2  photo-electron direction ($SELECT-PHOTOELECTRON-DIRECTION) of a
//           photo-electron of total energy E: out = {cos theta}
//   kind 3  pair production:                  out = {electron total energy, positron total energy}
//   kind 4  Moller, electron of total energy E: out = {fraction of the kinetic energy to the delta ray}
//   kind 5  Bhabha, positron of total energy E: out = {fraction of the kinetic energy to the electron,
//           before the swap that keeps the larger share on the positron}
//   kind 6  bremsstrahlung, electron of total energy E: out = {photon energy}
//   kind 7  Rayleigh scattering, photon of energy E: out = {cos theta}
//   kind 8  two-photon annihilation in flight, positron of total energy E:
//           out = {energy fraction of the first photon}
// out has 3 values per interaction (unused ones 0).
int oracle_sample_interaction(oracle_handle *h, int kind, int med, double E, long long n, uint32_t seed,
                              double *out) {
    Tally T;
    Run R;
    R.O = &h->O; R.T = &T; R.ranmar = false; R.seed = seed;
    if (med < 0 || med >= (int)h->O.H.media.size()) return 1;
    const Medium &m = h->O.H.media[med];
    for (long long i = 0; i < n; ++i) {
        Particle p;
        p.hist = (uint32_t)i; p.sid = 0; p.n = 0; p.cache_blk = -1; p.wt = 1;
        p.x = p.y = p.z = 0; p.u = 0; p.v = 0; p.w = 1; p.ir = 0;
        p.iq = kind == 2 ? -1 : 0;
        p.E = E;
        double *o = out + 3 * i;
        o[0] = o[1] = o[2] = 0;
        if (kind == 0 || kind == 1) {
            Particle el;
            double uj = compton(R, p, m, el, kind == 1);
            o[0] = p.E / E; o[1] = p.w; o[2] = uj;
        } else if (kind == 2) {
            // the direction part of PHOTO for a photo-electron of total energy E
            double eelec = E, beta = std::sqrt((eelec - RM) * (eelec + RM)) / eelec, gamma = eelec / RM;
            double alpha = 0.5 * gamma - 0.5 + 1. / gamma, ratio = beta / alpha, costhe, sinth2, xi;
            while (true) {
                double rn = rnd(R, p);
                rn = 2. * rn - 1.;
                if (ratio <= 0.2) {
                    double fk = rn + 0.5 * ratio * (1. - rn) * (1. + rn);
                    if (gamma < 100) costhe = (beta + fk) / (1. + beta * fk);
                    else if (fk > 0) costhe = 1 - (1 - fk) * (gamma - 3) / (2 * (1 + fk) * (gamma - 1) * (gamma - 1) * (gamma - 1));
                    else costhe = (beta + fk) / (1. + beta * fk);
                    xi = (1 + beta * fk) * gamma * gamma;
                } else {
                    xi = gamma * gamma * (1. + alpha * (std::sqrt(1. + ratio * (2. * rn + ratio)) - 1.));
                    costhe = (1. - 1. / xi) / beta;
                }
                sinth2 = std::max(0., (1. - costhe) * (1. + costhe));
                double rn2 = rnd(R, p);
                if (!(rn2 > 0.5 * (1. + gamma) * sinth2 * xi / gamma)) break;
            }
            o[0] = costhe;
        } else if (kind == 3) {
            Particle second;
            pair(R, p, m, second);
            o[0] = p.iq < 0 ? p.E : second.E;
            o[1] = p.iq < 0 ? second.E : p.E;
        } else if (kind == 4) {   // Moller, electron of total energy E (E > thmoll)
            if (!(E > m.thmoll)) return 1;
            o[0] = moller_br(R, p, m, E - RM, E);
        } else if (kind == 5) {   // Bhabha, positron of total energy E (kinetic > te)
            if (!(E - RM > m.te)) return 1;
            o[0] = bhabha_br(R, p, m, E - RM);
        } else if (kind == 8) {   // annihilation in flight, positron of total energy E
            const double a = (E + RM) / RM, g = a - 1.0, t = g - 1.0;
            if (!(t > 0)) return 1;
            const double pp = std::sqrt(a * t), ep0 = 1.0 / (a + pp), wsamp = std::log((1.0 - ep0) / ep0);
            o[0] = annih_ep(R, p, a, ep0, wsamp);
        } else if (kind == 7) {   // Rayleigh, photon of energy E: out = {cos theta}
            PhotonCtx pc;
            pc.gle = std::log(E);
            pc.lgle = interval(pc.gle, m.ge1, m.ge0);
            pc.cohfac = 1;
            if (pc.lgle < 1 || pc.lgle > m.mge) return 1;
            double costhe, sinthe;
            rayleigh_sample(R, p, m, pc, costhe, sinthe);
            o[0] = costhe;
        } else if (kind == 6) {   // bremsstrahlung photon energy, electron of total energy E (kinetic > ap)
            const double ekin = E - RM;
            if (!(ekin > m.ap)) return 1;
            const int l = (E < 50.0) ? 0 : 2;
            o[0] = brems_k(R, p, m, E, ekin, std::log(ekin), l, l + 1);
        } else {
            return 1;
        }
    }
    return R.errors ? 2 : 0;
}

// Thresholds of medium `med` (HATCH, from PEGS4): out[3] = {te (the Moller
// and Bhabha delta-ray threshold, kinetic), thmoll (the Moller threshold,
// total energy), ap (the bremsstrahlung photon threshold)}, MeV.
int oracle_medium_thresholds(oracle_handle *h, int med, double *out) {
    if (med < 0 || med >= (int)h->O.H.media.size()) return 1;
    const Medium &m = h->O.H.media[med];
    out[0] = m.te; out[1] = m.thmoll; out[2] = m.ap;
    return 0;
}

// Composition of medium `med` (PEGS4): out[0] = number of elements n, then
// Z_i (n values) and atoms per molecule p_i (n values); out holds 1 + 2 nmax.
int oracle_medium_elements(oracle_handle *h, int med, int nmax, double *out) {
    if (med < 0 || med >= (int)h->O.H.media.size()) return 1;
    const Medium &m = h->O.H.media[med];
    if (m.nne > nmax) return 1;
    out[0] = m.nne;
    for (int i = 0; i < m.nne; ++i) { out[1 + i] = m.zelem[i]; out[1 + m.nne + i] = m.pz[i]; }
    return 0;
}

// Pair-production constants of medium `med` (HATCH, from PEGS4): out[51] =
// {dl1..dl6 for l = 0..7 (dl[k][l] at 8 k + l), delcm, bpar[0], bpar[1]}.
int oracle_medium_pair(oracle_handle *h, int med, double *out) {
    if (med < 0 || med >= (int)h->O.H.media.size()) return 1;
    const Medium &m = h->O.H.media[med];
    for (int k = 0; k < 6; ++k)
        for (int l = 0; l < 8; ++l) out[8 * k + l] = m.dl[k][l];
    out[48] = m.delcm; out[49] = m.bpar[0]; out[50] = m.bpar[1];
    return 0;
}

// The source particles of histories [first, first+n) as they enter the
// phantom: out[9 i ...] = {charge, kinetic energy, x, y, z, u, v, w, region}
// (region -1 for a particle that misses; its position is then the source's).
int oracle_sample_source(oracle_handle *h, long long first, long long n, uint32_t seed, double *out) {
    Tally T;
    Run R;
    R.O = &h->O; R.T = &T; R.ranmar = false; R.seed = seed;
    for (long long i = 0; i < n; ++i) {
        Particle p;
        source_particle(R, (uint32_t)(first + i), p);
        double *o = out + 9 * i;
        o[0] = p.iq; o[1] = p.iq == 0 ? p.E : p.E - RM;
        o[2] = p.x; o[3] = p.y; o[4] = p.z; o[5] = p.u; o[6] = p.v; o[7] = p.w; o[8] = p.ir;
    }
    return R.errors ? 1 : 0;
}

// HOWFARLESS transport (on != 0) in the current, homogeneous phantom: call
// after oracle_set_geometry.
int oracle_set_howfarless(oracle_handle *h, int on) {
    Oracle &O = h->O;
    O.hfl = on != 0;
    O.hfl_t0.clear();
    O.hfl_t1.clear();
    if (!O.hfl) return 0;
    double mindel = 1e30;
    for (int i = 0; i < O.G.nx; ++i) mindel = std::min(mindel, O.G.xb[i + 1] - O.G.xb[i]);
    for (int i = 0; i < O.G.ny; ++i) mindel = std::min(mindel, O.G.yb[i + 1] - O.G.yb[i]);
    for (int i = 0; i < O.G.nz; ++i) mindel = std::min(mindel, O.G.zb[i + 1] - O.G.zb[i]);
    for (const Medium &m : O.H.media) {
        std::vector<double> t0, t1;
        howfarless_tmxs(m, O.H.params, mindel, t0, t1);
        O.hfl_t0.push_back(t0);
        O.hfl_t1.push_back(t1);
    }
    return 0;
}

int oracle_set_source(oracle_handle *h, const egsgpu_source *s) {
    h->O.S.s = *s;
    double n = std::sqrt(s->dir[0] * s->dir[0] + s->dir[1] * s->dir[1] + s->dir[2] * s->dir[2]);
    for (int k = 0; k < 3; ++k) h->O.S.s.dir[k] = s->dir[k] / n;
    h->O.S.has_rot = false;
    for (double r : s->rot) h->O.S.has_rot |= r != 0;
    if (h->O.S.has_rot && s->shape != 2) return 1;
    if (s->shape == 2) {
        if (s->nphsp < 1 || !s->phsp || s->recycle < 0) return 1;
        h->O.S.phsp.assign(s->phsp, s->phsp + 7 * s->nphsp);
        h->O.S.s.phsp = nullptr;
    } else if (s->spectrum == 1) build_alias(h->O.S);
    return 0;
}

// Runs histories [first, first+n) in nbatch batches; threads > 1 splits each
// batch into contiguous history ranges (Philox mode only).
int oracle_run(oracle_handle *h, long long first, long long n, int nbatch, uint32_t seed, int use_ranmar,
               int threads) {
    std::atomic<int> errs{0};
    if (use_ranmar) threads = 1;
    if (threads < 1) threads = 1;
    long long per_batch = n / nbatch;
    for (int b = 0; b < nbatch; ++b) {
        long long b0 = first + b * per_batch, bn = (b == nbatch - 1) ? n - b * per_batch : per_batch;
        std::vector<Tally> tl(threads);
        for (auto &t : tl) { t.batch.assign(h->T.batch.size(), 0); t.log_esc = h->T.log_esc; }
        std::vector<std::thread> th;
        long long per = bn / threads;
        for (int t = 0; t < threads; ++t) {
            long long s0 = b0 + t * per, sn = (t == threads - 1) ? bn - t * per : per;
            th.emplace_back(run_range, &h->O, &tl[t], s0, sn, 0, seed, use_ranmar, 0, 0,
                            h->hist_buf.empty() ? nullptr : h->hist_buf.data(), h->hist_first, h->hist_n, &errs);
        }
        for (auto &t : th) t.join();
        for (size_t i = 0; i < h->T.batch.size(); ++i) {
            double d = 0;
            for (auto &t : tl) d += t.batch[i];
            h->T.sum[i] += d;
            h->T.sum2[i] += d * d;
        }
        for (auto &t : tl) {
            h->T.esc_log.insert(h->T.esc_log.end(), t.esc_log.begin(), t.esc_log.end());
            h->T.dep += t.dep; h->T.esc += t.esc; h->T.steps += t.steps;
            h->T.psteps += t.psteps; h->T.esteps += t.esteps; h->T.pushes += t.pushes;
            h->T.tsteps += t.tsteps; h->T.msdist_calls += t.msdist_calls;
        }
    }
    h->nhist += n;
    h->nbatch += nbatch;
    return errs.load() ? 6 : 0;
}

// Maximum charged-particle step in cm (smaxir, src/egsnrc.mortran:1179);
// smax <= 0 restores the default (no limit).
int oracle_set_smax(oracle_handle *h, double smax) {
    h->O.H.params.smaxir = smax > 0 ? smax : 1e10;
    return 0;
}

// Records every particle that leaves the phantom from now on (on != 0), or
// stops recording; either way the record is cleared.
int oracle_set_escape_log(oracle_handle *h, int on) {
    h->T.log_esc = on != 0;
    h->T.esc_log.clear();
    return 0;
}
// Number of recorded escapes; copies up to `max` records (ESC_REC doubles
// each, in history order) to out.
long long oracle_get_escapes(oracle_handle *h, double *out, long long max) {
    long long n = (long long)(h->T.esc_log.size() / ESC_REC);
    if (out && max > 0) std::copy(h->T.esc_log.begin(), h->T.esc_log.begin() + std::min(n, max) * ESC_REC, out);
    return n;
}

int oracle_set_history_tally(oracle_handle *h, long long first, long long n) {
    h->hist_first = first; h->hist_n = n;
    h->hist_buf.assign(n > 0 ? (size_t)n : 0, 0.0);
    return 0;
}
int oracle_get_history_tally(oracle_handle *h, double *out) {
    std::copy(h->hist_buf.begin(), h->hist_buf.end(), out);
    return 0;
}

int oracle_get_tallies(oracle_handle *h, double *sum, double *sum2, double *totals) {
    if (sum) std::copy(h->T.sum.begin(), h->T.sum.end(), sum);
    if (sum2) std::copy(h->T.sum2.begin(), h->T.sum2.end(), sum2);
    if (totals) {
        totals[0] = (double)h->nhist; totals[1] = h->nbatch; totals[2] = h->T.dep; totals[3] = h->T.esc;
        totals[4] = h->T.steps; totals[5] = h->T.psteps; totals[6] = h->T.esteps; totals[7] = h->T.pushes;
    }
    return 0;
}

// Known-answer helpers for the oracle's own generators.
void oracle_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) { philox10(ctr, key, out); }
void oracle_ranmar(int ixx, int jxx, long long n, double *out) {
    Ranmar r;
    r.init(ixx, jxx);
    for (long long i = 0; i < n; ++i) out[i] = r.get();
}
uint64_t oracle_child_sid(uint64_t sid, uint32_t n, uint32_t k) { return child_sid(sid, n, k); }

// Table probes for host-data-layer tests.
double oracle_kn_sigma0(double e) { return kn_sigma0(e); }
int oracle_photon_xsec(oracle_handle *h, int med, double e, double *out4) {
    const Medium &m = h->O.H.media[med];
    double gle = std::log(e);
    int l = interval(gle, m.ge1, m.ge0) - 1;
    out4[0] = m.gmfp1[l] * gle + m.gmfp0[l];
    out4[1] = m.gbr11[l] * gle + m.gbr10[l];
    out4[2] = m.gbr21[l] * gle + m.gbr20[l];
    out4[3] = m.cohe1[l] * gle + m.cohe0[l];
    return l;
}
int oracle_electron_xsec(oracle_handle *h, int med, double eke, double *out8) {
    const Medium &m = h->O.H.media[med];
    double elke = std::log(eke);
    int l = interval(elke, m.eke1, m.eke0) - 1;
    const std::vector<double> *c[16] = {&m.esig0, &m.esig1, &m.psig0, &m.psig1, &m.ededx0, &m.ededx1, &m.pdedx0, &m.pdedx1,
                                        &m.ebr10, &m.ebr11, &m.pbr10, &m.pbr11, &m.pbr20, &m.pbr21, &m.tmxs0, &m.tmxs1};
    for (int k = 0; k < 8; ++k) out8[k] = (*c[2 * k + 1])[l] * elke + (*c[2 * k])[l];
    return l;
}

}  // extern "C"
