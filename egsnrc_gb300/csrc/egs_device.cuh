// Device-side data layout and random numbers of the GB300 transport engine.
// Templated on the transport precision Real (float or double); tallies are
// always FP64.  The FP32 electron kernel can compute the residual range, the
// energy loss and the face distances of steps near voxel faces in FP64
// (egsgpu_config.fp64_near_faces; the `wide_*` routines of egs_transport.cu).
// Paths in comments are relative to the EGSnrc HEN_HOUSE directory.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace egsgpu {

constexpr double RM = 0.5109989461;   // src/egsnrc.macros:1140
constexpr int MXGE = 2000;
constexpr int NRAY = 100;
constexpr int MS_NL = 64, MS_NQ = 8, MS_NU = 32;
constexpr int MAXMED = 16;            // media per problem (constant-memory scalars)
constexpr int MAXNE = 12;             // elements per medium
constexpr int LOOP_CAP_DEFAULT = 100000;   // iterations of one rejection loop
constexpr int STEP_CAP_DEFAULT = 1 << 22;  // transport steps of one particle

// The caps are set from egsgpu_config before every run (egsgpu_config.loop_cap,
// .step_cap); a loop or particle that reaches one is abandoned and the run
// returns EGSGPU_ERR_LOOP.  Each translation unit (FP32, FP64 engine) has its
// own copy, in its namespace EGSGPU_TU.
#ifndef EGSGPU_TU
#define EGSGPU_TU tu32
#endif
namespace EGSGPU_TU {
__constant__ int c_loop_cap = LOOP_CAP_DEFAULT;
__constant__ int c_step_cap = STEP_CAP_DEFAULT;
}  // namespace EGSGPU_TU
#define LOOP_CAP (::egsgpu::EGSGPU_TU::c_loop_cap)
#define STEP_CAP (::egsgpu::EGSGPU_TU::c_step_cap)

// ------------------------------------------------------------- tables ----
// Per-medium scalars, one struct per medium in constant memory.
template <class Real>
struct MedScalars {
    Real rho, ae, ap, te, thmoll, blcc, xcc, eke0, eke1, ge0, ge1, esig_e, psig_e, log_ap, delcm,
        zbrang, lzbrang;
    Real dl[6][8];
    Real bpar[2];
    Real E_array0;
    int meke, n_shell, nne, sig_mono_e, sig_mono_p;
    int etab_off, gtab_off, shell_off, elem_off;
    float pz[MAXNE];
};

// Device pointers into the table blob.
template <class Real>
struct Tables {
    const Real *etab;     // [medium][meke][16]: esig0,esig1,psig0,psig1,ededx0,ededx1,pdedx0,pdedx1,
                          //                     ebr10,ebr11,pbr10,pbr11,pbr20,pbr21,tmxs0,tmxs1
    const Real *erange;   // [medium][meke][4]: E_array, range_ep0, range_ep1, pad
    const Real *gtab;     // [medium][MXGE][8]: gmfp0,gmfp1,gbr10,gbr11,gbr20,gbr21,cohe0,cohe1
    const Real *pmax;     // [medium][MXGE][2]
    const Real *ray;      // [medium][4][NRAY]: xgrid, fcum, b_array, c_array
    const int *ray_i;     // [medium][NRAY] (1-based bins)
    const Real *shell;    // [shell_off + i][4]: eno (alias threshold), be (rm units), Jo, erfJo
    const int *shell_at;  // [shell_off + i]: alias bin (1-based)
    const Real *elem;     // [elem_off + k][96]: edge_a[16] b[16] c[16] d[16] energies[16] binding[6] iprob[6] | nedge
    const Real *ms;       // [MS_NL*MS_NQ*MS_NU][3]: ums, fms, wms
    const int *ms_i;      // [MS_NL*MS_NQ*MS_NU]
    Real dllambi, dqmsi;
    int nmed;
    // run parameters
    Real ecut, pcut, skindepth, smaxir;
};

// ------------------------------------------------------------ geometry ----
// One XYZ phantom.  Voxel indices are global: a run of several phantoms
// places phantom k's voxels at [voff, voff + nx*ny*nz) of shared medium,
// density and tally arrays (voff = 0 for a single phantom).
template <class Real>
struct Geom {
    int nx, ny, nz, nxy;
    const Real *xb, *yb, *zb;
    const uint8_t *med;   // global arrays, indexed by the global voxel index
    const Real *rhor;
    Real bt, hbt;         // boundary tolerance (egs++/egs_functions.h:80-88)
    int voff;             // global index of this phantom's first voxel
    // voxel-index decoding without integer division: n / nx and n / nxy as
    // (umulhi(n, m) + n) >> l with m, l from fast_divisor (exact for n < 2^31)
    uint32_t mnx, mnxy;
    int lnx, lnxy;
};
__device__ inline int fdiv(int n, uint32_t m, int l) {
    return (int)((__umulhi((uint32_t)n, m) + (uint32_t)n) >> l);
}

// ------------------------------------------------------------- source ----
struct Source {
    int charge, shape, spectrum, nbins;
    double pos[3], xmin, xmax, ymin, ymax, dir[3], energy;
    const double *edges;  // device
    const double *wi;     // device alias weights
    const int *bin;       // device alias bins
    long long nphsp;      // shape 2: phase-space particles (device, 7 floats each)
    const float *phsp;
    int recycle;
    int has_rot;          // shape 2: rotate the particles by rot (row-major)
    double rot[9];
};

// -------------------------------------------------------------- queues ----
// Structure-of-arrays particle queue in HBM.  Photon queues ignore iq.
// A particle parked mid-flight (a warp gave it up when its lanes ran low)
// carries its transport state: st = 0 fresh; photons st = 1 with aux[0] the
// remaining mean free paths; electrons st = 1 (new step sequence) or
// st = 2 | 4*compute_tstep with aux = {demfp, total_de, total_tstep, sig0}.
template <class Real>
struct Queue {
    Real *x, *y, *z, *u, *v, *w, *E, *wt;
    int *ir;
    int8_t *iq;
    uint32_t *hist, *n;
    unsigned long long *sid;
    uint8_t *st;
    Real *aux0, *aux1, *aux2, *aux3;
    unsigned int *count;  // device counter (pushes)
    unsigned int capacity;
};

// ---------------------------------------------------------------- RNG ----
// Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) keyed by (seed, history)
// with counter (block, stream id lo, stream id hi, 0).
__host__ __device__ inline void philox10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0,
                                         uint32_t k1, uint32_t out[4]) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
#ifdef __CUDA_ARCH__
        uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
        uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
#else
        uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0, hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
#endif
        uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

__host__ __device__ inline uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
__host__ __device__ inline uint64_t child_sid(uint64_t sid, uint32_t n, uint32_t k) {
    return mix64(sid + 0x9E3779B97F4A7C15ull * (1 + (((uint64_t)n) << 3) + k));
}

// One Philox block, kept out of line: the generator is called from about a
// hundred places in the transport kernels and inlining its ten rounds at each
// would multiply the kernels' instruction footprint.
// (internal linkage: each translation unit of the engine has its own copy;
// host-callable so that the generator's window logic can be checked on a CPU)
static __host__ __device__ __noinline__ uint4 philox_block(uint32_t b, uint32_t s0, uint32_t s1, uint32_t k0,
                                                           uint32_t k1);

// The generator keeps a window of the stream's next four Philox blocks
// (block b in slot b & 3; `next` is one past the highest block held).  A
// draw refills only when its block is missing.  The transport loops call
// ahead(k) where the warp is converged, so that the blocks the lanes will
// need for the coming step are computed there, by all lanes together, instead
// of at whichever draw site a lane's counter happens to cross into a new block
// (the lanes' counters are out of phase, so in a lazily filled stream almost
// every draw site runs the ten Philox rounds for one or two of its lanes).
// The numbers are the same either way: the window only decides when a block
// is computed.  A copy holds the stream position but not the window, so
// particle copies stay small and a copy never reads blocks it did not compute.
struct Rng {
    uint32_t seed, hist, n, next;
    uint64_t sid;
    alignas(16) uint32_t c[16];
    Rng() = default;
    __host__ __device__ Rng(const Rng &o) : seed(o.seed), hist(o.hist), n(o.n), next(0), sid(o.sid) {}
    __host__ __device__ Rng &operator=(const Rng &o) {
        seed = o.seed; hist = o.hist; n = o.n; sid = o.sid; next = 0;
        return *this;
    }
    __host__ __device__ void init(uint32_t s, uint32_t h, uint64_t id, uint32_t n0) {
        seed = s; hist = h; sid = id; n = n0; next = 0;
    }
    __host__ __device__ inline void fill(uint32_t b) {
        reinterpret_cast<uint4 *>(c)[b & 3u] = philox_block(b, (uint32_t)sid, (uint32_t)(sid >> 32), seed, hist);
    }
    // make the blocks holding the next k numbers (1 <= k <= 13) present.  The ten
    // rounds are inlined here (one copy per transport loop): a call to the
    // shared out-of-line block from this site measured 10-20% slower.
    __host__ __device__ inline void ahead(uint32_t k) {
        const uint32_t b0 = n >> 2, b1 = (n + k - 1) >> 2;
        uint32_t b = next > b0 ? next : b0;
        for (; b <= b1; ++b) {
            uint32_t o[4];
            philox10(b, (uint32_t)sid, (uint32_t)(sid >> 32), 0u, seed, hist, o);
            reinterpret_cast<uint4 *>(c)[b & 3u] = make_uint4(o[0], o[1], o[2], o[3]);
        }
        if (b > next) next = b;
    }
    // Out of line (as is azimuth): the electron step loop is larger than the
    // instruction caches, and one shared copy of the draw for its ~30 call
    // sites measured 20-40% faster than inlined copies, even though the
    // generator state then lives in local memory around each call.  Sites that
    // take two numbers in a row call u2 (one call instead of two: +3% on
    // electron-dominated phantoms).
    __host__ __device__ __noinline__ float u() { return draw(); }
    __host__ __device__ __noinline__ float2 u2() {
        float a = draw();
        return make_float2(a, draw());
    }
    __host__ __device__ inline float draw() {
        const uint32_t b = n >> 2;
        // present: b < next, and b >= next - 4 since ahead() never runs more
        // than three blocks past the current one
        if (b >= next) { fill(b); next = b + 1; }
        const uint32_t x = c[n & 15u];
        ++n;
        // (x >> 9) + 0.5 scaled by 2^-23: exact in FP32 and FP64, in (0,1)
        return ((float)(x >> 9) + 0.5f) * (1.0f / 8388608.0f);
    }
};
// Uniform in (0,1) with 23 random bits: the same value in FP32 and FP64.
template <class Real>
__device__ inline Real urand(Rng &r) { return (Real)r.u(); }
// two consecutive uniforms in one call (the same numbers as two urand calls)
__device__ inline float2 urand2(Rng &r) { return r.u2(); }

// --------------------------------------------------------- math shims ----
// FP32 transport uses the SFU-based intrinsics; FP64 uses the full-precision
// library functions (so that the FP64 build tracks the CPU oracle).
__device__ inline float dlog(float x) { return __logf(x); }
__device__ inline double dlog(double x) { return log(x); }
__device__ inline float dexp(float x) { return __expf(x); }
__device__ inline double dexp(double x) { return exp(x); }
__device__ inline float dsqrt(float x) { return sqrtf(x); }
__device__ inline double dsqrt(double x) { return sqrt(x); }
__device__ inline float dcos(float x) { return cosf(x); }
__device__ inline double dcos(double x) { return cos(x); }
template <class T> __device__ inline T dmin(T a, T b) { return a < b ? a : b; }
template <class T> __device__ inline T dmax(T a, T b) { return a > b ? a : b; }
template <class T> __device__ inline T dabs(T a) { return a < 0 ? -a : a; }

}  // namespace egsgpu
