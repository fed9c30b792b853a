// egs_gpu_app: runs an egs++ voxel-dose input (EGS_XYZGeometry +
// EGS_ParallelBeam + EGS_DoseScoring) on the GPU engine through the C ABI.
//
//   egs_gpu_app -i input.egsinp -p 521icru [-o name] [--data DIR] [--precision 32|64]
//
// It plays the role of an egs++ application built with APP_MAIN
// (egs++/egs_application.h:1218-1226) for this path: the input blocks are the
// ones egs_app reads (run control, geometry definition, media, source
// definition, MC transport parameter, rng definition, ausgab object
// definition), the PEGS4 file is given with -p, and the dose goes to
// <name>.3ddose in the egs_dose_scoring format, normalised as EGS_DoseScoring
// normalises it: the dose per history times ncase / F, F the source's fluence
// (ncase / area for a parallel beam; for a phase-space source the incident
// particles of the original simulation times the fraction of the file read).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>
#include <chrono>
#include <unistd.h>
#include <libgen.h>

#include "egs_input.h"
#include "egsgpu.h"

using egsin::Item;

static int fail(const std::string &m) {
    std::fprintf(stderr, "egs_gpu_app: %s\n", m.c_str());
    return 1;
}

static std::string exe_dir() {
    char buf[4096];
    ssize_t n = readlink("/proc/self/exe", buf, sizeof(buf) - 1);
    if (n <= 0) return ".";
    buf[n] = 0;
    return std::string(dirname(buf));
}

struct Phantom {
    int nx = 0, ny = 0, nz = 0;
    std::vector<double> xb, yb, zb, rho_abs, rhor;
    std::vector<int32_t> med;
    std::vector<std::string> media;
    bool abs_density = false;
};

static bool planes(const Item *g, const char *p, const char *s, std::vector<double> &b) {
    if (g->has(p)) { b = Item::numbers(g->get(p)); return b.size() >= 2; }
    if (g->has(s)) {   // "x-slabs = first, width, count"
        auto v = Item::numbers(g->get(s));
        if (v.size() != 3 || v[2] < 1) return false;
        b.clear();
        for (int i = 0; i <= (int)v[2]; ++i) b.push_back(v[0] + i * v[1]);
        return true;
    }
    return false;
}

// Phase-space sources: EGS_PhspSource (egs++/sources/egs_phsp_source/
// egs_phsp_source.cpp:196-290 input, :364-470 reading and rejection) and
// IAEA_PhspSource (egs++/sources/iaea_phsp_source/iaea_phsp_source.cpp:226-308
// input, :310-470).  The file is read by egsgpu_read_phsp.  A rejected particle
// keeps its place in the list with weight 0, as the reference hands it to the
// application with wt = 0.  Rejection: the particle type ('particle type' =
// electrons, photons, positrons, all or charged), the 'cutout' rectangle
// (x_min x_max y_min y_max), the 'weight window' (wmin wmax) on the stored
// weight divided by the number of uses (the sign of an egsphsp weight is the
// sign of w and takes part, as in the reference), and, for egsphsp files,
// LATCH bit 31 and the LATCH filter.
// The IAEA source hands out LATCH 0, so bit 31 never rejects there.  Recycling
// ('reuse photons/electrons', or 'recycle ...') must be the same number for
// both.  Returns the plane z of the particles in *zplane.
static bool load_phsp_source(const Item *s, bool iaea, std::vector<float> &phsp, int &recycle, double &zplane,
                             double &incident, std::string &err) {
    const std::string path = s->get(iaea ? "iaea phase space file" : "phase space file");
    egsgpu_phsp_info info;
    if (egsgpu_read_phsp(path.c_str(), 0, 0, &info, nullptr, nullptr, nullptr)) {
        err = egsgpu_last_error(nullptr);
        return false;
    }
    phsp.resize((size_t)info.n * 7);
    std::vector<uint32_t> latch((size_t)info.n);
    if (egsgpu_read_phsp(path.c_str(), 0, info.n, &info, phsp.data(), latch.data(), nullptr)) {
        err = egsgpu_last_error(nullptr);
        return false;
    }
    if (!(info.zmin == info.zmax)) {
        err = path + ": the particles are not on one plane z = const";
        return false;
    }
    zplane = info.zmin;
    const std::string pt = egsin::norm(s->get("particle type", "all"));
    const int want = pt == "photons" ? 0 : pt == "electrons" ? -1 : pt == "positrons" ? 1 : pt == "charged" ? 2 : 3;
    if (want == 3 && pt != "all") { err = "unknown particle type '" + pt + "'"; return false; }
    auto cut = Item::numbers(s->get("cutout", ""));
    auto win = Item::numbers(s->get("weight window", ""));
    auto rec = [&](const std::string &what) {   // 'reuse ...', else 'recycle ...'
        return (int)std::max(0.0, s->num("reuse " + what, s->num("recycle " + what, 0)));
    };
    const int rp = rec("photons"), re = rec("electrons");
    if (rp != re) { err = "different recycle numbers for photons and electrons are not supported"; return false; }
    recycle = rp;
    // LATCH filter (egs_phsp_source.cpp:226-252, :446-518): 'filter type = 0' with
    // 'latch setting = b1 b2', two strings of 0/1 for LATCH bits 0, 1, ...: a particle
    // is rejected unless it has one of the bits set to 1 in b1 (when b1 has any), or
    // when it has one of the bits set to 1 in b2, which count on from where b1 ends.
    // More than 29 bits in all leaves the filter off, as in the reference.
    uint32_t filter1 = 0, filter2 = 0;
    if (s->has("filter type") && s->has("latch setting")) {
        const auto ft = Item::numbers(s->get("filter type"));
        const auto ls = Item::words(s->get("latch setting"));
        if (!ft.empty() && ft[0] != 0) {
            err = "only 'filter type = 0' is supported (types 1-3 set no filter bits in egs++ either)";
            return false;
        }
        if (iaea) {
            err = "LATCH filters need the egsphsp LATCH: IAEA_PhspSource hands out LATCH 0";
            return false;
        }
        const std::string b1 = ls.size() > 0 ? ls[0] : "", b2 = ls.size() > 1 ? ls[1] : "";
        if (b1.size() + b2.size() <= 29) {
            for (size_t i = 0; i < b1.size(); ++i)
                if (b1[i] == '1') filter1 |= 1u << i;
            for (size_t j = 0; j < b2.size(); ++j)
                if (b2[j] == '1') filter2 |= 1u << (b1.size() + j);
        }
    }
    for (size_t i = 0, k = 0; i < phsp.size(); i += 7, ++k) {
        const float q = phsp[i];
        bool keep = want == 3 || (want == 2 ? q != 0 : q == (float)want);
        if (cut.size() == 4 && (phsp[i + 2] < cut[0] || phsp[i + 2] > cut[1] || phsp[i + 3] < cut[2] ||
                                phsp[i + 3] > cut[3]))
            keep = false;
        if (win.size() == 2) {
            const double wt = (iaea ? std::fabs(phsp[i + 6]) : phsp[i + 6]) / (recycle + 1.0);
            if (wt < win[0] || wt > win[1]) keep = false;
        }
        if (!iaea && (latch[k] & 0x80000000u)) keep = false;
        if ((filter1 && !(latch[k] & filter1)) || (latch[k] & filter2)) keep = false;
        if (!keep) phsp[i + 6] = phsp[i + 6] < 0 ? -0.0f : 0.0f;
    }
    incident = info.incident;
    std::printf("phase space: %lld particles, %.0f incident histories\n", info.n, info.incident);
    return true;
}

// The rotation of an egs++ transformation block
// (EGS_AffineTransform::getTransformation, egs++/egs_transformations.cpp:44-108,
// matrices egs++/egs_transformations.h:153-200, 303-355), row-major into R:
// 'rotation vector' = v is the matrix EGS_RotationMatrix(v) builds, rotY(cos t,
// -sin t) rotZ(cos p, sin p) for the polar and azimuthal angles t, p of v;
// 'rotation' = phi theta is R_z(phi) R_x(theta), alpha beta gamma is
// R_x(alpha) R_y(beta) R_z(gamma), vx vy vz phi is R1^T R_z(phi) R1 with R1 the
// matrix of v, nine numbers the matrix itself.  Returns 1 with R filled, 0 when
// the block has no rotation, -1 (message in err) for a zero vector.
namespace {
struct M3 {
    double a[9];
    M3 operator*(const M3 &o) const {
        M3 r;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j)
                r.a[3 * i + j] = a[3 * i] * o.a[j] + a[3 * i + 1] * o.a[3 + j] + a[3 * i + 2] * o.a[6 + j];
        return r;
    }
    M3 t() const { return {{a[0], a[3], a[6], a[1], a[4], a[7], a[2], a[5], a[8]}}; }
};
M3 m_eye() { return {{1, 0, 0, 0, 1, 0, 0, 0, 1}}; }
M3 m_rx(double c, double s) { return {{1, 0, 0, 0, c, s, 0, -s, c}}; }
M3 m_ry(double c, double s) { return {{c, 0, -s, 0, 1, 0, s, 0, c}}; }
M3 m_rz(double c, double s) { return {{c, s, 0, -s, c, 0, 0, 0, 1}}; }
bool m_of_vector(double x, double y, double z, M3 &r) {
    double sinz = x * x + y * y, norm = sinz + z * z;
    if (norm < 1e-10) return false;
    norm = std::sqrt(norm);
    if (sinz > 1e-10) {
        sinz = std::sqrt(sinz);
        r = m_ry(z / norm, -sinz / norm) * m_rz(x / sinz, y / sinz);
    } else if (z < 0) {
        r = m_rx(std::cos(M_PI), std::sin(M_PI));
    } else {
        r = m_eye();
    }
    return true;
}
}  // namespace

static int egs_rotation(const Item *t, double *R, std::string &err) {
    auto fail_rot = [&](const char *what) {
        err = std::string("transformation: ") + what;   // egs++ stops with a fatal error here
        return -1;
    };
    M3 m = m_eye();
    auto v = Item::numbers(t->get("rotation vector", ""));
    auto r = Item::numbers(t->get("rotation", ""));
    if (v.size() == 3) {
        if (!m_of_vector(v[0], v[1], v[2], m)) return fail_rot("a rotation vector of length 0");
    } else if (r.size() == 2) {
        m = m_rz(std::cos(r[0]), std::sin(r[0])) * m_rx(std::cos(r[1]), std::sin(r[1]));
    } else if (r.size() == 3) {
        m = m_rx(std::cos(r[0]), std::sin(r[0])) * m_ry(std::cos(r[1]), std::sin(r[1])) *
            m_rz(std::cos(r[2]), std::sin(r[2]));
    } else if (r.size() == 4) {
        M3 r1;
        if (!m_of_vector(r[0], r[1], r[2], r1)) return fail_rot("a rotation axis of length 0");
        m = r1.t() * m_rz(std::cos(r[3]), std::sin(r[3])) * r1;
    } else if (r.size() == 9) {
        for (int k = 0; k < 9; ++k) m.a[k] = r[k];
    } else {
        return 0;
    }
    for (int k = 0; k < 9; ++k) R[k] = m.a[k];
    return 1;
}

static const char *MEDCH = "123456789ABCDEFGHIJKLMNOPQRSTUVWXYZabcdefghijklmnopqrstuvwxyz";

static bool read_egsphant(const std::string &path, Phantom &P, std::string &err) {
    std::ifstream f(path);
    if (!f) { err = "cannot open egsphant file " + path; return false; }
    int nmed;
    f >> nmed;
    P.media.resize(nmed);
    for (auto &m : P.media) f >> m;
    for (int i = 0; i < nmed; ++i) { double e; f >> e; }
    f >> P.nx >> P.ny >> P.nz;
    P.xb.resize(P.nx + 1); P.yb.resize(P.ny + 1); P.zb.resize(P.nz + 1);
    for (auto &v : P.xb) f >> v;
    for (auto &v : P.yb) f >> v;
    for (auto &v : P.zb) f >> v;
    size_t nv = (size_t)P.nx * P.ny * P.nz;
    P.med.resize(nv);
    for (int k = 0; k < P.nz; ++k)
        for (int j = 0; j < P.ny; ++j) {
            std::string row;
            f >> row;
            if ((int)row.size() < P.nx) { err = "short medium row in " + path; return false; }
            for (int i = 0; i < P.nx; ++i) {
                const char *c = std::strchr(MEDCH, row[i]);
                if (!c || c - MEDCH >= nmed) { err = "bad medium character in " + path; return false; }
                P.med[(size_t)k * P.nx * P.ny + (size_t)j * P.nx + i] = (int32_t)(c - MEDCH);
            }
        }
    P.rho_abs.resize(nv);
    for (auto &v : P.rho_abs) f >> v;
    if (!f) { err = "truncated egsphant file " + path; return false; }
    P.abs_density = true;
    return true;
}

int main(int argc, char **argv) {
    std::string input, pegs, out, data = exe_dir() + "/data";
    int precision = 32;
    for (int i = 1; i < argc; ++i) {
        std::string a = argv[i];
        auto next = [&]() { return i + 1 < argc ? std::string(argv[++i]) : std::string(); };
        if (a == "-i") input = next();
        else if (a == "-p") pegs = next();
        else if (a == "-o") out = next();
        else if (a == "--data") data = next();
        else if (a == "--precision") precision = std::atoi(next().c_str());
        else return fail("unknown option " + a);
    }
    if (input.empty() || pegs.empty()) return fail("usage: egs_gpu_app -i input -p pegsfile [-o name] [--data dir]");
    if (input.find('.') == std::string::npos) input += ".egsinp";
    if (out.empty()) {
        out = input.substr(0, input.rfind('.'));
    }
    std::string pegs_file = pegs;
    if (pegs_file.find('/') == std::string::npos) pegs_file = data + "/" + pegs_file;
    if (pegs_file.find(".pegs4dat") == std::string::npos) pegs_file += ".pegs4dat";

    std::string err;
    auto root = egsin::parse(input, err);
    if (!root) return fail(err);

    // ---- run control (egs++/egs_run_control.cpp:90-110) ----
    const Item *rc = root->block("run control");
    long long ncase = rc ? (long long)rc->num("ncase", 1024) : 1024;
    int nbatch = rc ? (int)rc->num("nbatch", 10) : 10;

    // ---- transport parameters (egs++/egs_advanced_application.cpp:482-562) ----
    egsgpu_config cfg;
    egsgpu_default_config(&cfg);
    cfg.precision = precision;
    if (const Item *mc = root->block("MC transport parameter")) {
        cfg.ecut = mc->num("Global ECUT", cfg.ecut);
        cfg.pcut = mc->num("Global PCUT", cfg.pcut);
        cfg.estepe = mc->num("ESTEPE", cfg.estepe);
        cfg.ximax = mc->num("XImax", cfg.ximax);
        cfg.skindepth = mc->num("Skin depth for BCA", cfg.skindepth);
        cfg.smax = mc->num("Global Smax", cfg.smax);
        if (mc->has("Boundary crossing algorithm")) {
            const std::string b = egsin::norm(mc->get("Boundary crossing algorithm"));
            if (b == "presta-i") cfg.bca_algorithm = 1;
            else if (b != "exact")
                return fail("'Boundary crossing algorithm = " + mc->get("Boundary crossing algorithm") +
                            "' is not supported (EXACT or PRESTA-I)");
        }
        struct Fixed { const char *key, *value; } fixed[] = {
            {"Electron-step algorithm", "presta-ii"},
            {"Spin effects", "off"}, {"Brems angular sampling", "km"}, {"Brems cross sections", "bh"},
            {"Pair angular sampling", "simple"}, {"Pair cross sections", "bh"}, {"Triplet production", "off"},
            {"Electron impact ionization", "off"}, {"Photonuclear attenuation", "off"},
            {"Photon cross sections", "xcom"}, {"Bound Compton scattering", "norej"},
            {"Rayleigh scattering", "on"}, {"Atomic relaxations", "on"}, {"Photoelectron angular sampling", "on"}};
        for (auto &fx : fixed)
            if (mc->has(fx.key) && egsin::norm(mc->get(fx.key)) != fx.value)
                return fail(std::string("'") + fx.key + " = " + mc->get(fx.key) +
                            "' is not supported (this engine implements " + fx.value + ")");
    }

    // ---- geometry (EGS_XYZGeometry, egs_nd_geometry.cpp:1160-1260) ----
    const Item *gd = root->block("geometry definition");
    if (!gd) return fail("no geometry definition");
    std::string gname = gd->get("simulation geometry");
    const Item *g = nullptr;
    for (auto *b : gd->blocks("geometry"))
        if (egsin::norm(b->get("name")) == egsin::norm(gname)) g = b;
    if (!g) return fail("simulation geometry '" + gname + "' not defined");
    if (egsin::norm(g->get("type")) != "egs_xyzgeometry")
        return fail("only EGS_XYZGeometry is supported on this path");
    Phantom P;
    if (g->has("egsphant file")) {
        if (!read_egsphant(g->get("egsphant file"), P, err)) return fail(err);
    } else {
        if (!planes(g, "x-planes", "x-slabs", P.xb) || !planes(g, "y-planes", "y-slabs", P.yb) ||
            !planes(g, "z-planes", "z-slabs", P.zb))
            return fail("XYZ geometry needs x/y/z planes or slabs");
        P.nx = (int)P.xb.size() - 1; P.ny = (int)P.yb.size() - 1; P.nz = (int)P.zb.size() - 1;
        size_t nv = (size_t)P.nx * P.ny * P.nz;
        P.med.assign(nv, 0);
        P.rhor.assign(nv, 1.0);
        const Item *mi = g->block("media input");
        if (!mi) return fail("geometry has no media input");
        P.media = Item::words(mi->get("media"));
        // 'set medium = i j', '= i1 i2 j' or '= i1 i2 j step' (egs_base_geometry.cpp:787-811)
        for (auto &v : mi->all("set medium")) {
            auto n = Item::numbers(v);
            int a, b, m, step = 1;
            if (n.size() == 2) { a = b = (int)n[0]; m = (int)n[1]; }
            else if (n.size() >= 3) { a = (int)n[0]; b = (int)n[1]; m = (int)n[2]; if (n.size() > 3) step = (int)n[3]; }
            else return fail("bad 'set medium' input");
            if (m < 0 || m >= (int)P.media.size()) return fail("'set medium' refers to an undefined medium");
            for (int r = std::max(a, 0); r <= std::min<long long>(b, (long long)nv - 1); r += std::max(step, 1)) P.med[r] = m;
        }
        for (auto &v : mi->all("set relative density")) {
            auto n = Item::numbers(v);
            int a = (int)(n[0] + 0.1), b = n.size() == 3 ? (int)(n[1] + 0.1) : a;
            double r = n.back();
            for (int k = std::max(a, 0); k <= std::min<long long>(b, (long long)nv - 1); ++k) P.rhor[k] = r;
        }
        for (auto &v : g->all("set relative density")) {
            auto n = Item::numbers(v);
            int a = (int)(n[0] + 0.1), b = n.size() == 3 ? (int)(n[1] + 0.1) : a;
            for (int k = std::max(a, 0); k <= std::min<long long>(b, (long long)nv - 1); ++k) P.rhor[k] = n.back();
        }
    }

    // ---- source (EGS_ParallelBeam; egs_base_source.cpp:46, egs_parallel_beam.cpp:43) ----
    const Item *sd = root->block("source definition");
    if (!sd) return fail("no source definition");
    std::string sname = sd->get("simulation source");
    const Item *s = nullptr;
    for (auto *b : sd->blocks("source"))
        if (egsin::norm(b->get("name")) == egsin::norm(sname)) s = b;
    if (!s) return fail("simulation source '" + sname + "' not defined");
    egsgpu_source src;
    std::memset(&src, 0, sizeof(src));
    // EGS_TransformedSource (egs++/sources/egs_transformed_source): the inner
    // source's particles are rotated by R and shifted by the translation
    double shift[3] = {0, 0, 0}, rot[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    bool rotated = false;
    if (egsin::norm(s->get("library")) == "egs_transformed_source") {
        const Item *t = s->block("transformation");
        if (t) {
            auto v = Item::numbers(t->get("translation", "0 0 0"));
            if (v.size() == 3)
                for (int k = 0; k < 3; ++k) shift[k] = v[k];
            std::string rerr;
            const int rc = egs_rotation(t, rot, rerr);
            if (rc < 0) return fail(rerr);
            rotated = rc > 0;
        }
        std::string inner = s->get("source name");
        const Item *in = nullptr;
        for (auto *b : sd->blocks("source"))
            if (egsin::norm(b->get("name")) == egsin::norm(inner)) in = b;
        if (!in) return fail("source '" + inner + "' not defined");
        s = in;
    }
    std::vector<float> phsp;
    std::vector<double> edges, weights;   // the source points into these until egsgpu_set_source
    // EGS_DoseScoring scales the dose per history by ncase / F, F the source's
    // fluence (egs_dose_scoring.cpp:309-320): ncase / area for EGS_ParallelBeam
    // (egs_parallel_beam.h:157), so the factor is the shape's area (1 for a point)
    double norm_e = 1;
    std::string lib = egsin::norm(s->get("library"));
    if (lib == "egs_phsp_source" || lib == "iaea_phsp_source") {
        double zplane = 0, incident = 0;
        std::string perr;
        if (!load_phsp_source(s, lib == "iaea_phsp_source", phsp, src.recycle, zplane, incident, perr))
            return fail(perr);
        // fluence F = Pinc * Nread / Nparticle (egs_phsp_source.h:153-156): Nread
        // records are read for ncase histories, each used recycle + 1 times
        const double nread = (double)((ncase + src.recycle) / (src.recycle + 1));
        if (incident > 0 && nread > 0) norm_e = (double)ncase / (incident * nread / (double)(phsp.size() / 7));
        src.shape = 2;
        src.nphsp = (long long)(phsp.size() / 7);
        src.phsp = phsp.data();
        // the file's plane z0: R (x, y, z0) + t = R (x, y, 0) + (t + z0 R e_z)
        for (int k = 0; k < 3; ++k) src.pos[k] = shift[k] + zplane * rot[3 * k + 2];
        src.dir[2] = 1;
        if (rotated)
            for (int k = 0; k < 9; ++k) src.rot[k] = rot[k];
    } else if (lib != "egs_parallel_beam")
        return fail("only egs_parallel_beam, egs_phsp_source and iaea_phsp_source sources are supported");
    if (rotated && lib != "egs_phsp_source" && lib != "iaea_phsp_source")
        return fail("rotated sources are supported for phase-space sources only");
    if (lib == "egs_parallel_beam") {
    src.charge = (int)s->num("charge", 0);
    auto dir = Item::numbers(s->get("direction", "0 0 1"));
    for (int k = 0; k < 3; ++k) src.dir[k] = k < (int)dir.size() ? dir[k] : 0;
    const Item *sh = s->block("shape");
    if (!sh) return fail("source has no shape");
    std::string stype = egsin::norm(sh->get("type"));
    double tr[3] = {0, 0, 0};
    if (const Item *t = sh->block("transformation")) {
        auto v = Item::numbers(t->get("translation", "0 0 0"));
        for (int k = 0; k < 3 && k < (int)v.size(); ++k) tr[k] = v[k];
    }
    if (stype == "point") {
        auto p = Item::numbers(sh->get("position", "0 0 0"));
        src.shape = 0;
        for (int k = 0; k < 3; ++k) src.pos[k] = (k < (int)p.size() ? p[k] : 0) + tr[k];
    } else if (stype == "rectangle") {
        auto r = Item::numbers(sh->get("rectangle"));
        if (r.size() != 4) return fail("rectangle needs x1 y1 x2 y2");
        src.shape = 1;
        src.xmin = std::min(r[0], r[2]) + tr[0]; src.xmax = std::max(r[0], r[2]) + tr[0];
        src.ymin = std::min(r[1], r[3]) + tr[1]; src.ymax = std::max(r[1], r[3]) + tr[1];
        norm_e = (src.xmax - src.xmin) * (src.ymax - src.ymin);
        src.pos[2] = tr[2];
    } else return fail("shape type '" + sh->get("type") + "' is not supported");
    const Item *sp = s->block("spectrum");
    if (!sp) return fail("source has no spectrum");
    std::string sptype = egsin::norm(sp->get("type"));
    if (sptype == "monoenergetic") {
        src.spectrum = 0;
        src.energy = sp->num("energy", 0);
    } else if (sptype == "tabulated spectrum") {
        edges = Item::numbers(sp->get("energies"));
        weights = Item::numbers(sp->get("probabilities"));
        int mode = (int)sp->num("spectrum mode", sp->num("spectrum type", 1));
        if (mode != 1 || edges.size() != weights.size() + 1 || weights.empty())
            return fail("tabulated spectra must be histograms (mode 1: N+1 energies, N probabilities)");
        src.spectrum = 1;
        src.nbins = (int)weights.size();
        src.edges = edges.data();
        src.weights = weights.data();
    } else return fail("spectrum type '" + sp->get("type") + "' is not supported");
    for (int k = 0; k < 3; ++k) src.pos[k] += shift[k];
    src.xmin += shift[0]; src.xmax += shift[0]; src.ymin += shift[1]; src.ymax += shift[1];
    }
    // ---- engine (after the whole input has been read: input errors need no GPU) ----
    egsgpu_handle *h = nullptr;
    int st = egsgpu_create(&cfg, &h);
    if (st) return fail("egsgpu_create failed with status " + std::to_string(st));
    std::vector<const char *> names;
    for (auto &m : P.media) names.push_back(m.c_str());
    if ((st = egsgpu_load_media(h, data.c_str(), pegs_file.c_str(), names.data(), (int)names.size())))
        return fail(egsgpu_last_error(h));
    if (P.abs_density) {   // relative density = mass density / PEGS4 density
        P.rhor.resize(P.rho_abs.size());
        for (size_t i = 0; i < P.rho_abs.size(); ++i) {
            double info[4];
            egsgpu_get_medium(h, P.med[i], info);
            P.rhor[i] = P.rho_abs[i] / info[0];
        }
    }
    if ((st = egsgpu_set_xyz_geometry(h, P.nx, P.ny, P.nz, P.xb.data(), P.yb.data(), P.zb.data(), P.med.data(),
                                      P.rhor.data())))
        return fail(egsgpu_last_error(h));

    if ((st = egsgpu_set_source(h, &src))) return fail(egsgpu_last_error(h));

    uint32_t seed = 1;
    if (const Item *rng = root->block("rng definition")) {
        auto v = Item::numbers(rng->get("initial seeds", "1"));
        if (!v.empty()) seed = (uint32_t)v[0];
    }

    auto t0 = std::chrono::steady_clock::now();
    if ((st = egsgpu_run(h, 0, ncase, nbatch, seed, nullptr))) return fail(egsgpu_last_error(h));
    double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();

    size_t nv = (size_t)P.nx * P.ny * P.nz;
    std::vector<double> dose(nv), sig(nv);
    double tot[8];
    egsgpu_get_dose(h, dose.data(), sig.data());
    egsgpu_get_tallies(h, nullptr, nullptr, tot);
    std::printf("histories %lld in %d batches, %.3f s (%.4g histories/s)\n", ncase, nbatch, dt, ncase / dt);
    std::printf("deposited %.6g MeV, escaped %.6g MeV per history\n", tot[2] / ncase, tot[3] / ncase);
    std::printf("dose normalisation ncase / fluence = %.6g\n", norm_e);

    // .3ddose (egs_dose_scoring.cpp:416-480)
    std::string fn = out + ".3ddose";
    FILE *f = std::fopen(fn.c_str(), "w");
    if (!f) return fail("cannot write " + fn);
    std::fprintf(f, "%d %d %d\n", P.nx, P.ny, P.nz);
    for (auto *b : {&P.xb, &P.yb, &P.zb}) {
        for (double v : *b) std::fprintf(f, "%g ", (float)v);
        std::fprintf(f, "\n");
    }
    for (size_t i = 0; i < nv; ++i) std::fprintf(f, "%g ", (float)(dose[i] * norm_e));
    std::fprintf(f, "\n");
    for (size_t i = 0; i < nv; ++i) std::fprintf(f, "%g ", (float)(dose[i] > 0 ? sig[i] / dose[i] : 1.0));
    std::fprintf(f, "\n");
    std::fclose(f);
    std::printf("wrote %s\n", fn.c_str());
    egsgpu_destroy(h);
    return 0;
}
