// Host data layer: the cold initialisation that EGSnrc performs in HATCH.
//
// Every table the transport kernels read is built here, in FP64, from the
// same data files EGSnrc reads:
//   * the PEGS4 per-medium block                 (egsnrc.mortran:2013-2221)
//   * XCOM photon cross sections on a 2000-bin
//     log grid, bound-Compton corrected          (egs_init_user_photon :7973-8280)
//   * Rayleigh form-factor sampling tables       (egs_init_rayleigh :8284, prepare_rayleigh_data :8593)
//   * derived electron tables (range, tmxs,
//     fictitious cross-section maxima)           (mscati :2750-2979)
//   * the q^(2+) multiple-scattering surface     (init_ms_SR :3267-3305)
//   * Compton shell data + alias table           (init_compton :2442-2594)
//   * photo-absorption edges and shell probs     (EDGSET :6312, egs_init_user_photon :8105-8120)
//   * bremsstrahlung / pair rejection constants  (fix_brems :2322-2413, egsnrc.macros:1981-1994)
// All paths in comments are relative to the EGSnrc HEN_HOUSE directory.
#pragma once
#include <string>
#include <vector>
#include <cstdint>

namespace egs {

constexpr double RM = 0.5109989461;          // egsnrc.macros:1140
constexpr double RMT2 = 2 * RM;
constexpr double RMSQ = RM * RM;
constexpr int MXGE = 2000;                   // egsnrc.macros:195
constexpr int MXRAYFF = 100;                 // egsnrc.macros:205
constexpr int RAYCDFSIZE = 100;              // egsnrc.macros:206
constexpr int MS_NL = 64, MS_NQ = 8, MS_NU = 32;   // egsnrc.macros:851-860
constexpr double LAMBMIN_MS = 1.0, LAMBMAX_MS = 1e5, QMIN_MS = 1e-3, QMAX_MS = 0.5;
constexpr int MXSHELL = 6, MXINTER = 5;      // egsnrc.macros:492-493
constexpr int MXEDGE = 16;                   // max photo_cs edge intervals per element
constexpr int MXMDSH = 200;                  // egsnrc.macros:445

// Per-element photo-absorption data (EDGSET, egsnrc.mortran:6312-6425).
struct ElementPhoto {
    int Z = 0;
    int edge_number = 0;
    double edge_a[MXEDGE] = {}, edge_b[MXEDGE] = {}, edge_c[MXEDGE] = {},
           edge_d[MXEDGE] = {}, edge_energies[MXEDGE] = {};
    double binding[MXSHELL] = {};            // MeV, shells K,L1,L2,L3,...
    double interaction_prob[MXSHELL] = {};   // [5] = 1.01 as in EDGSET
};

// Global Compton shell list from incoh.data (init_compton :2442-2490).
struct ComptonShells {
    std::vector<int> iz, shn, ne;
    std::vector<double> Jo, be, erfJo;       // be in units of RM
};

struct Medium {
    std::string name;
    // composition
    double rho = 0;
    int nne = 0;
    std::vector<double> zelem, wa, pz, rhoz;
    // thresholds
    double rlc = 0, ae = 0, ap = 0, ue = 0, up = 0, te = 0, thmoll = 0;
    int meke = 0, mge = 0, irayl = 0;
    // brems / pair constants: dl[k][l], k = 0..5 -> dl1..dl6, l = 0..7
    double dl[6][8] = {};
    double delcm = 0, alphi[2] = {}, bpar[2] = {}, delpos[2] = {};
    double log_ap = 0, zbrang = 0, lzbrang = 0;
    // electron tables (cm units after HATCH scaling)
    double xr0 = 0, teff0 = 0, blcc = 0, xcc = 0;
    double eke0 = 0, eke1 = 0;
    std::vector<double> esig0, esig1, psig0, psig1, ededx0, ededx1, pdedx0, pdedx1,
        ebr10, ebr11, pbr10, pbr11, pbr20, pbr21, tmxs0, tmxs1;
    // derived by mscati
    std::vector<double> E_array, range_ep0, range_ep1;
    double esig_e = 0, psig_e = 0, expeke1 = 0;
    bool sig_ismonotone[2] = {false, false};
    // photon tables (rebuilt from XCOM)
    double ebinda = 0, ge0 = 0, ge1 = 0;
    std::vector<double> gmfp0, gmfp1, gbr10, gbr11, gbr20, gbr21, cohe0, cohe1;
    // Rayleigh sampling
    double xgrid[MXRAYFF] = {}, fcum[MXRAYFF] = {}, b_array[MXRAYFF] = {}, c_array[MXRAYFF] = {};
    int i_array[RAYCDFSIZE] = {};
    std::vector<double> pmax0, pmax1;
    // Compton shells of this medium (alias table over shells)
    int n_shell = 0;
    std::vector<double> eno_array;           // alias thresholds (1-based semantics kept)
    std::vector<int> eno_atbin_array, shell_array;   // shell_array: index into ComptonShells
    // elements (index into Hatch::elements) in PEGS order
    std::vector<int> elem_index;
};

// Transport parameters of the physics profile (egs_set_defaults and the egs++
// "MC transport parameter" block; egs_advanced_application.cpp:482-562).
struct TransportParams {
    double ecut = 0.521, pcut = 0.010;        // total energy for e-, MeV
    double estepe = 0.25, ximax = 0.5;       // egsnrc.macros:2265, :2260
    double skindepth_for_bca = 3.0;          // egsnrc.macros:2256; PRESTA-I with <= 1e-4: the
                                             // old PRESTA default, set by hatch()
    bool exact_bca = true;                   // BCA: EXACT, or PRESTA-I (false)
    int transport_algorithm = 0;             // 0 = PRESTA-II
    bool spin_effects = false;               // spinms.data absent
    int ibcmp = 3;                           // bound Compton norej
    int iraylr = 1, iedgfl = 1, iphter = 1;  // Rayleigh, relaxations, Sauter
    int ibrdst = 1, iprdst = 1;              // KM brems angle, simple pair angle
    double smaxir = 1e10;                    // egsnrc.macros:2271 ($MAX-SMAX)
};

struct Hatch {
    TransportParams params;
    std::vector<Medium> media;
    std::vector<ElementPhoto> elements;      // only elements used by the media
    ComptonShells shells;
    // MS q-surface (init_ms_SR), index [i][j][k] -> (i*MS_NQ + j)*MS_NU + k
    std::vector<double> ums, fms, wms;
    std::vector<int> ims;
    double dllambi = 0, dqmsi = 0;
    double max_binding_energy = 0;           // largest shell binding energy over all media (MeV)
};

// Build every table for the named media. `data_dir` holds the staged data
// files; `pegs_file` is the PEGS4 material file. Returns 0 on success, a
// positive error class otherwise, with a message in `err`.
int hatch(const std::string &data_dir, const std::string &pegs_file,
          const std::vector<std::string> &media, const TransportParams &params,
          Hatch &out, std::string &err);

// Klein-Nishina total cross section per electron (egsnrc.mortran:8728-8745).
double kn_sigma0(double e);

// Largest condensed-history step for DOSXYZnrc's HOWFARLESS transport in a
// homogeneous phantom (dosxyznrc.mortran modify_tmxs, :4795-4840): the
// estepe / ximax step at every node of the electron energy grid, but never
// below half the smallest voxel dimension `mindel` (cm).  Returns the
// piecewise-linear coefficients (t0 + t1 * log E per bin) of medium m.
void howfarless_tmxs(const Medium &m, const TransportParams &p, double mindel, std::vector<double> &t0,
                     std::vector<double> &t1);

}  // namespace egs
