// Host data layer: restatement of EGSnrc's HATCH table construction.
// Paths in comments are relative to the EGSnrc HEN_HOUSE directory.
#include "egs_hatch.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <map>
#include <sstream>

namespace egs {

namespace {

// Line-oriented numeric reader with Fortran record semantics: a read of n
// values consumes whole lines and drops the unread remainder of the last one.
struct LineReader {
    std::vector<std::string> lines;
    size_t pos = 0;
    bool ok = true;

    bool open(const std::string &path) {
        std::ifstream f(path);
        if (!f) return false;
        std::string s;
        while (std::getline(f, s)) lines.push_back(s);
        return true;
    }
    bool eof() const { return pos >= lines.size(); }
    void skip(size_t n = 1) { pos += n; }
    std::vector<double> read(size_t n) {
        std::vector<double> v;
        v.reserve(n);
        while (v.size() < n) {
            if (pos >= lines.size()) { ok = false; break; }
            const char *p = lines[pos++].c_str();
            while (v.size() < n) {
                char *end;
                while (*p == ' ' || *p == '\t' || *p == ',' || *p == '\r') ++p;
                if (!*p) break;
                double x = std::strtod(p, &end);
                if (end == p) { ok = false; return v; }
                v.push_back(x);
                p = end;
            }
        }
        return v;
    }
    std::vector<double> read_line() {
        std::vector<double> v;
        if (pos >= lines.size()) { ok = false; return v; }
        const char *p = lines[pos++].c_str();
        while (true) {
            char *end;
            while (*p == ' ' || *p == '\t' || *p == ',' || *p == '\r') ++p;
            if (!*p) break;
            double x = std::strtod(p, &end);
            if (end == p) break;
            v.push_back(x);
            p = end;
        }
        return v;
    }
};

std::string trim(const std::string &s) {
    size_t a = s.find_first_not_of(" \t\r");
    size_t b = s.find_last_not_of(" \t\r");
    return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
}

double field_after(const std::string &line, const std::string &key, bool &ok) {
    size_t p = line.find(key);
    if (p == std::string::npos) { ok = false; return 0; }
    return std::strtod(line.c_str() + p + key.size(), nullptr);
}

// Fortran INT() of the PWLF interval expression, 1-based.
inline int set_interval(double x, double c1, double c0) { return (int)(c1 * x + c0); }

// Per-element XCOM-format data: ln(E) and ln(sigma) pairs.
struct XData { std::vector<double> e, f; };

bool read_xcom(const std::string &path, std::vector<XData> &out) {
    LineReader r;
    if (!r.open(path)) return false;
    out.assign(101, XData());
    for (int iz = 1; iz <= 100; ++iz) {
        auto nd = r.read(1);
        if (!r.ok) return false;
        int ndat = (int)nd[0];
        auto v = r.read(2 * (size_t)ndat);
        if (!r.ok) return false;
        out[iz].e.resize(ndat);
        out[iz].f.resize(ndat);
        for (int k = 0; k < ndat; ++k) { out[iz].e[k] = v[2 * k]; out[iz].f[k] = v[2 * k + 1]; }
    }
    return true;
}

// egsi_get_data (egsnrc.mortran:8748-8825): accumulate pz-weighted element
// cross sections on the medium's log-energy grid. flag 0: photo/Rayleigh,
// 1: pair (threshold 2m), 2: triplet (threshold 4m).
bool get_data(int flag, const std::vector<XData> &xd, int n, const std::vector<int> &zs,
              const std::vector<double> &pzs, double ge1, double ge0, std::vector<double> &data,
              std::string &err) {
    data.assign(n, 0.0);
    for (size_t i = 0; i < zs.size(); ++i) {
        int iz = zs[i];
        std::vector<double> et, ft;
        double eth = 0;
        if (flag == 0) {
            et = xd[iz].e; ft = xd[iz].f;
        } else {
            eth = (flag == 1) ? 2 * RM : 4 * RM;
            et.push_back(std::log(eth)); ft.push_back(0);
            for (size_t k = 0; k < xd[iz].e.size(); ++k) {
                et.push_back(xd[iz].e[k]);
                ft.push_back(xd[iz].f[k] - 3 * std::log(1 - eth / std::exp(xd[iz].e[k])));
            }
            ft[0] = ft[1];
        }
        int ndat = (int)et.size();
        for (int k = 1; k <= n; ++k) {
            double gle = (k - ge0) / ge1, e = std::exp(gle), sig;
            if (gle < et[0] || gle >= et[ndat - 1]) {
                if (flag == 0) {
                    char b[200];
                    std::snprintf(b, sizeof b, "photon energy %g outside data range of element %d", e, iz);
                    err = b;
                    return false;
                }
                sig = (gle < et[0]) ? 0.0 : std::exp(ft[ndat - 1]);
            } else {
                int kk = 0;
                for (kk = 0; kk < ndat - 1; ++kk)
                    if (gle >= et[kk] && gle < et[kk + 1]) break;
                double p = (gle - et[kk]) / (et[kk + 1] - et[kk]);
                sig = std::exp(p * ft[kk + 1] + (1 - p) * ft[kk]);
            }
            if (flag != 0 && e > eth) sig *= std::pow(1 - eth / e, 3);
            data[k - 1] += pzs[i] * sig;
        }
    }
    return true;
}

double fcoulc(double Z) {   // egsnrc.mortran:2417-2426
    const double fine = 137.03604;
    double asq = Z / fine;
    asq = asq * asq;
    return asq * (1.0 / (1.0 + asq) + 0.20206 + asq * (-0.0369 + asq * (0.0083 + asq * (-0.002))));
}

double xsif(double Z) {     // egsnrc.mortran:2428-2440
    const double alrad[4] = {5.31, 4.79, 4.74, 4.71};
    const double alradp[4] = {6.144, 5.621, 5.805, 5.924};
    if (Z <= 4) {
        int iz = (int)Z;
        return alradp[iz - 1] / (alrad[iz - 1] - fcoulc(Z));
    }
    return std::log(1194.0 * std::pow(Z, -0.666667)) / (std::log(184.15 * std::pow(Z, -0.33333)) - fcoulc(Z));
}

int read_pegs4(const std::string &path, const std::vector<std::string> &names,
               std::vector<Medium> &media, std::string &err) {
    LineReader r;
    if (!r.open(path)) { err = "cannot open PEGS4 file " + path; return 2; }
    media.assign(names.size(), Medium());
    std::vector<bool> found(names.size(), false);
    size_t nfound = 0;
    while (!r.eof() && nfound < names.size()) {
        const std::string &hdr = r.lines[r.pos++];
        if (hdr.compare(0, 8, " MEDIUM=") != 0) continue;
        // 24-character name match (egsnrc.mortran:2017-2029)
        std::string nm = trim(hdr.substr(8, std::min<size_t>(24, hdr.size() - 8)));
        size_t im = names.size();
        for (size_t k = 0; k < names.size(); ++k)
            if (!found[k] && trim(names[k]) == nm) { im = k; break; }
        if (im == names.size()) continue;
        Medium &m = media[im];
        m.name = nm;
        bool ok = true;
        const std::string &l2 = r.lines[r.pos++];
        m.rho = field_after(l2, "RHO=", ok);
        m.nne = (int)field_after(l2, "NE=", ok);
        if (!ok || m.nne < 1) { err = "bad composition line for medium " + nm; return 3; }
        for (int ie = 0; ie < m.nne; ++ie) {
            const std::string &le = r.lines[r.pos++];
            m.zelem.push_back(field_after(le, ",Z=", ok));
            m.wa.push_back(field_after(le, ",A=", ok));
            m.pz.push_back(field_after(le, ",PZ=", ok));
            m.rhoz.push_back(field_after(le, ",RHOZ=", ok));
        }
        if (!ok) { err = "bad element line for medium " + nm; return 3; }
        auto t = r.read(5);
        m.rlc = t[0]; m.ae = t[1]; m.ap = t[2]; m.ue = t[3]; m.up = t[4];
        m.te = m.ae - RM;
        m.thmoll = m.te * 2 + RM;
        auto sz = r.read_line();
        if (sz.size() < 8) { err = "bad size line for medium " + nm; return 3; }
        m.meke = (int)sz[3];
        m.mge = (int)sz[1];
        m.irayl = (int)sz[7];
        auto dl = r.read(36);
        for (int i = 0; i < 6; ++i)
            for (int k = 0; k < 6; ++k) m.dl[k][i] = dl[i * 6 + k];
        auto bp = r.read(7);
        m.delcm = bp[0];
        m.alphi[0] = bp[1]; m.bpar[0] = bp[2]; m.delpos[0] = bp[3];
        m.alphi[1] = bp[4]; m.bpar[1] = bp[5]; m.delpos[1] = bp[6];
        auto ei = r.read(4);
        m.xr0 = ei[0]; m.teff0 = ei[1]; m.blcc = ei[2]; m.xcc = ei[3];
        auto ek = r.read(2);
        m.eke0 = ek[0]; m.eke1 = ek[1];
        auto et = r.read(16 * (size_t)m.meke);
        std::vector<double> *cols[16] = {&m.esig0, &m.esig1, &m.psig0, &m.psig1, &m.ededx0, &m.ededx1,
                                         &m.pdedx0, &m.pdedx1, &m.ebr10, &m.ebr11, &m.pbr10, &m.pbr11,
                                         &m.pbr20, &m.pbr21, &m.tmxs0, &m.tmxs1};
        for (auto c : cols) c->resize(m.meke);
        for (int i = 0; i < m.meke; ++i)
            for (int c = 0; c < 16; ++c) (*cols[c])[i] = et[16 * (size_t)i + c];
        auto pb = r.read(3);
        m.ebinda = pb[0]; m.ge0 = pb[1]; m.ge1 = pb[2];
        r.read(6 * (size_t)m.mge);   // PEGS4 photon tables: replaced by the XCOM rebuild
        if (m.irayl == 1) {
            auto ngr = r.read(1);
            r.read(2);
            r.read(2 * (size_t)ngr[0]);
            r.read(2 * (size_t)m.mge);
        }
        if (!r.ok) { err = "premature end of PEGS4 data for medium " + nm; return 3; }
        // distance-unit scaling, DUNIT = 1 cm (egsnrc.mortran:2198-2221)
        double dfact = m.rlc, dfacti = 1.0 / dfact;
        for (int i = 0; i < m.meke; ++i) {
            m.esig0[i] *= dfacti; m.esig1[i] *= dfacti; m.psig0[i] *= dfacti; m.psig1[i] *= dfacti;
            m.ededx0[i] *= dfacti; m.ededx1[i] *= dfacti; m.pdedx0[i] *= dfacti; m.pdedx1[i] *= dfacti;
            m.tmxs0[i] *= dfact; m.tmxs1[i] *= dfact;
        }
        m.teff0 *= dfact;
        m.blcc *= dfacti;
        m.xcc *= std::sqrt(dfacti);
        found[im] = true;
        ++nfound;
    }
    if (nfound < names.size()) {
        err = "media not found in PEGS4 file:";
        for (size_t k = 0; k < names.size(); ++k)
            if (!found[k]) err += " " + names[k];
        return 3;
    }
    return 0;
}

}  // namespace

void howfarless_tmxs(const Medium &m, const TransportParams &p, double mindel, std::vector<double> &t0,
                     std::vector<double> &t1) {
    const int neke = m.meke;
    t0.assign(neke, 0.0);
    t1.assign(neke, 0.0);
    // the estepe / ximax step length at energy e with stopping power dedx
    auto step = [&](double e, double dedx) {
        double p2 = e * (e + 2 * RM), beta2 = p2 / (p2 + RM * RM);
        double chi_a2 = m.xcc / (4 * p2 * m.blcc);
        double estepx = 2 * p2 * beta2 * dedx / e / m.xcc / (std::log(1 + 1. / chi_a2) * (1 + chi_a2) - 1);
        estepx = std::min(estepx * p.ximax, p.estepe);
        return std::max(estepx * e / dedx, mindel / 2);
    };
    double eil = (1 - m.eke0) / m.eke1;
    double si = step(std::exp(eil), m.ededx1[0] * eil + m.ededx0[0]);
    for (int i = 1; i <= neke - 1; ++i) {
        double elke = (i + 1 - m.eke0) / m.eke1;
        double sip1 = step(std::exp(elke), m.ededx1[i] * elke + m.ededx0[i]);
        t1[i - 1] = (sip1 - si) * m.eke1;
        t0[i - 1] = sip1 - t1[i - 1] * elke;
        si = sip1;
    }
    t0[neke - 1] = t0[neke - 2];
    t1[neke - 1] = t1[neke - 2];
}

double kn_sigma0(double e) {   // egs_KN_sigma0, egsnrc.mortran:8728-8745
    const double con = 0.1274783851;
    double ko = e / RM;
    if (ko < 0.01) return 8. * con / 3. * (1 - ko * (2 - ko * (5.2 - 13.3 * ko))) / RM;
    double c1 = 1. / (ko * ko), c2 = 1. - 2 * (1 + ko) * c1, c3 = (1 + 2 * ko) * c1;
    double eps2 = 1, eps1 = 1. / (1 + 2 * ko);
    return (c1 * (1. / eps1 - 1. / eps2) + c2 * std::log(eps2 / eps1) + eps2 * (c3 + 0.5 * eps2) -
            eps1 * (c3 + 0.5 * eps1)) / e * con;
}

int hatch(const std::string &dir, const std::string &pegs_file, const std::vector<std::string> &names,
          const TransportParams &params, Hatch &H, std::string &err) {
    H = Hatch();
    H.params = params;
    const std::string d = dir.empty() || dir.back() == '/' ? dir : dir + "/";
    int rc = read_pegs4(pegs_file, names, H.media, err);
    if (rc) return rc;
    const int nmed = (int)H.media.size();

    // $INITIALIZE-BREMS-ANGLE (egsnrc.macros:1981-1994)
    for (auto &m : H.media) {
        double zb = 0, pzn = 0;
        for (int ie = 0; ie < m.nne; ++ie) { zb += m.pz[ie] * m.zelem[ie] * (m.zelem[ie] + 1.0); pzn += m.pz[ie]; }
        m.zbrang = 8.116224e-05 * std::pow(zb / pzn, 1. / 3.);
        m.lzbrang = -std::log(m.zbrang);
    }

    // ---- XCOM photon cross sections (egs_init_user_photon :7973-8280) ----
    std::vector<XData> xphoto, xpair, xtrip, xray;
    if (!read_xcom(d + "xcom_photo.data", xphoto) || !read_xcom(d + "xcom_pair.data", xpair) ||
        !read_xcom(d + "xcom_triplet.data", xtrip) || !read_xcom(d + "xcom_rayleigh.data", xray)) {
        err = "cannot read XCOM data files in " + d;
        return 2;
    }
    // binding energies from the edges of the photo-absorption data (:8105-8122)
    std::vector<std::vector<double>> binding(101, std::vector<double>(31, 0.0));
    for (int iz = 1; iz <= 100; ++iz) {
        const auto &e = xphoto[iz].e;
        int k = 0;
        for (int j = (int)e.size() - 1; j >= 1; --j) {
            if (e[j] - e[j - 1] < 1e-5) {
                ++k;
                if (k <= 30) binding[iz][k] = std::exp(e[j]);
            }
        }
    }
    // bound Compton correction data (compton_sigma.data)
    LineReader cs;
    if (!cs.open(d + "compton_sigma.data")) { err = "cannot open compton_sigma.data"; return 2; }
    auto csh = cs.read(3);
    double bc_emin = csh[0], bc_emax = csh[1];
    int bc_ne = (int)csh[2];
    std::vector<std::vector<double>> bc_z(101);
    for (int iz = 1; iz <= 100 && cs.ok; ++iz) bc_z[iz] = cs.read(bc_ne);
    if (!cs.ok) { err = "bad compton_sigma.data"; return 2; }
    double bc_dle = std::log(bc_emax / bc_emin) / (bc_ne - 1);
    // atomic form factors (pgs4form.dat), aff[i + 100*(Z-1)]
    LineReader ffr;
    if (!ffr.open(d + "pgs4form.dat")) { err = "cannot open pgs4form.dat"; return 2; }
    auto xval = ffr.read(MXRAYFF);
    auto aff = ffr.read((size_t)MXRAYFF * 100);
    if (!ffr.ok) { err = "bad pgs4form.dat"; return 2; }

    for (int im = 0; im < nmed; ++im) {
        Medium &m = H.media[im];
        m.mge = MXGE;
        const int nge = MXGE;
        m.ge1 = (nge - 1) / std::log(m.up / m.ap);
        m.ge0 = 1 - m.ge1 * std::log(m.ap);
        double sumZ = 0, sumA = 0;
        std::vector<std::pair<double, double>> zp;
        for (int i = 0; i < m.nne; ++i) {
            sumZ += m.pz[i] * m.zelem[i];
            sumA += m.pz[i] * m.wa[i];
            zp.push_back({m.zelem[i], m.pz[i]});
        }
        std::stable_sort(zp.begin(), zp.end(), [](auto &a, auto &b) { return a.first < b.first; });
        std::vector<int> zs;
        std::vector<double> pzs;
        for (auto &p : zp) { zs.push_back((int)(p.first + 0.5)); pzs.push_back(p.second); }
        double con2 = m.rho / (sumA * 1.6605655);
        std::vector<double> sph, sray, spair, strip;
        if (!get_data(0, xphoto, nge, zs, pzs, m.ge1, m.ge0, sph, err) ||
            !get_data(0, xray, nge, zs, pzs, m.ge1, m.ge0, sray, err) ||
            !get_data(1, xpair, nge, zs, pzs, m.ge1, m.ge0, spair, err) ||
            !get_data(2, xtrip, nge, zs, pzs, m.ge1, m.ge0, strip, err))
            return 3;
        std::vector<double> bc(bc_ne, 0.0);
        for (size_t i = 0; i < zs.size(); ++i)
            for (int j = 0; j < bc_ne; ++j) bc[j] += pzs[i] * zp[i].first * bc_z[zs[i]][j];
        for (int j = 0; j < bc_ne; ++j) bc[j] = std::log(bc[j] / sumZ);

        // ---- Rayleigh form factors, IAM (egs_init_rayleigh :8380-8395) ----
        double ff[MXRAYFF];
        for (int i = 0; i < MXRAYFF; ++i) {
            double s = 0;
            m.xgrid[i] = xval[i];
            for (int j = 0; j < m.nne; ++j) {
                double a = aff[i + (size_t)MXRAYFF * ((int)m.zelem[j] - 1)];
                s += m.pz[j] * a * a;
            }
            ff[i] = std::sqrt(s);
        }
        if (m.xgrid[0] < 1e-6) m.xgrid[0] = 1e-4;
        // prepare_rayleigh_data (:8593-8726)
        {
            const int ndat = MXRAYFF, ne = m.mge, ncbin = RAYCDFSIZE;
            double *x = m.xgrid, *f = ff;
            double emin = std::exp((1 - m.ge0) / m.ge1), emax = std::exp((m.mge - m.ge0) / m.ge1);
            for (int i = 0; i < ndat; ++i) if (f[i] == 0.0) f[i] = 1e-30;
            double b_arr[MXRAYFF] = {};
            double sum0 = 0;
            m.fcum[0] = 0;
            for (int i = 0; i < ndat - 1; ++i) {
                double b = std::log(f[i + 1] / f[i]) / std::log(x[i + 1] / x[i]);
                b_arr[i] = b;
                double x1 = x[i], x2 = x[i + 1], p1 = std::pow(x1, 2 * b), p2 = std::pow(x2, 2 * b);
                sum0 += f[i] * f[i] * (x2 * x2 * p2 - x1 * x1 * p1) / ((1 + b) * p1);
                m.fcum[i + 1] = sum0;
            }
            std::vector<double> pe(ne);
            double dle = std::log(emax / emin) / (ne - 1);
            int i = 0;   // 0-based
            for (int j = 0; j < ne; ++j) {
                double e = emin * std::exp(dle * j), xmax = 20.607544 * 2 * e / RM;
                int k;
                for (k = i; k < ndat - 1; ++k)
                    if (xmax >= x[k] && xmax < x[k + 1]) break;
                i = k;
                double b = b_arr[i], x1 = x[i], x2 = xmax;
                double p1 = std::pow(x1, 2 * b), p2 = std::pow(x2, 2 * b);
                pe[j] = m.fcum[i] + f[i] * f[i] * (x2 * x2 * p2 - x1 * x1 * p1) / ((1 + b) * p1);
            }
            m.i_array[ncbin - 1] = i + 1;   // stored 1-based like the reference
            double anorm = 1.0 / std::sqrt(pe[ne - 1]), anorm1 = 1.005 / pe[ne - 1], anorm2 = 1.0 / pe[ne - 1];
            for (int j = 0; j < ne; ++j) { pe[j] *= anorm1; if (pe[j] > 1) pe[j] = 1; }
            for (int j = 0; j < ndat; ++j) {
                f[j] *= anorm;
                m.fcum[j] *= anorm2;
                m.c_array[j] = (1 + b_arr[j]) / ((x[j] * f[j]) * (x[j] * f[j]));
            }
            double dw = 1.0 / (ncbin - 1), xold = x[0];
            int ibin = 0;
            double b = b_arr[0], pow_x1 = std::pow(x[0], 2 * b);
            m.i_array[0] = 1;
            for (int ii = 1; ii < ncbin - 1; ++ii) {
                double w = dw;
                for (int guard = 0; guard < 100000; ++guard) {
                    double x1 = xold, x2 = x[ibin + 1];
                    double t = x1 * x1 * std::pow(x1, 2 * b), pow_x2 = std::pow(x2, 2 * b);
                    double aux = f[ibin] * f[ibin] * (x2 * x2 * pow_x2 - t) / ((1 + b) * pow_x1);
                    if (aux > w) {
                        xold = std::exp(std::log(t + w * (1 + b) * pow_x1 / f[ibin] / f[ibin]) / (2 + 2 * b));
                        m.i_array[ii] = ibin + 1;
                        break;
                    }
                    w -= aux;
                    xold = x2;
                    ++ibin;
                    b = b_arr[ibin];
                    pow_x1 = std::pow(xold, 2 * b);
                }
            }
            for (int j = 0; j < ndat; ++j) m.b_array[j] = 0.5 / (1 + b_arr[j]);
            m.pmax0.assign(ne, 0);
            m.pmax1.assign(ne, 0);
            for (int k = 0; k < ne - 1; ++k) {
                double gle = (k + 1 - m.ge0) / m.ge1;
                m.pmax1[k] = (pe[k + 1] - pe[k]) * m.ge1;
                m.pmax0[k] = pe[k] - m.pmax1[k] * gle;
            }
            m.pmax0[ne - 1] = m.pmax0[ne - 2];
            m.pmax1[ne - 1] = m.pmax1[ne - 2];
        }

        // ---- attenuation, branching and Rayleigh-fraction tables ----
        m.gmfp0.assign(nge, 0); m.gmfp1.assign(nge, 0);
        m.gbr10.assign(nge, 0); m.gbr11.assign(nge, 0);
        m.gbr20.assign(nge, 0); m.gbr21.assign(nge, 0);
        m.cohe0.assign(nge, 0); m.cohe1.assign(nge, 0);
        double gmfp_old = 0, gbr1_old = 0, gbr2_old = 0, cohe_old = 0, gle = 0;
        double gmfp = 0, gbr1 = 0, gbr2 = 0, cohe = 0;
        for (int i = 1; i <= nge; ++i) {
            gle = (i - m.ge0) / m.ge1;
            double e = std::exp(gle);
            double sig_kn = sumZ * kn_sigma0(e);
            double bcf;
            if (e <= bc_emin) bcf = std::exp(bc[0]);
            else if (e < bc_emax) {
                double aj = 1 + std::log(e / bc_emin) / bc_dle;
                int j = (int)aj;
                aj -= j;
                bcf = std::exp(bc[j - 1] * (1 - aj) + bc[j] * aj);
            } else bcf = 1;
            sig_kn *= bcf;
            double sig_p = spair[i - 1] + strip[i - 1];
            double sigma = sig_kn + sig_p + sph[i - 1];
            gmfp = 1 / (sigma * con2);
            gbr1 = sig_p / sigma;
            gbr2 = gbr1 + sig_kn / sigma;
            cohe = sigma / (sray[i - 1] + sigma);
            if (i > 1) {
                m.gmfp1[i - 2] = (gmfp - gmfp_old) * m.ge1; m.gmfp0[i - 2] = gmfp - m.gmfp1[i - 2] * gle;
                m.gbr11[i - 2] = (gbr1 - gbr1_old) * m.ge1; m.gbr10[i - 2] = gbr1 - m.gbr11[i - 2] * gle;
                m.gbr21[i - 2] = (gbr2 - gbr2_old) * m.ge1; m.gbr20[i - 2] = gbr2 - m.gbr21[i - 2] * gle;
                m.cohe1[i - 2] = (cohe - cohe_old) * m.ge1; m.cohe0[i - 2] = cohe - m.cohe1[i - 2] * gle;
            }
            gmfp_old = gmfp; gbr1_old = gbr1; gbr2_old = gbr2; cohe_old = cohe;
        }
        m.gmfp1[nge - 1] = m.gmfp1[nge - 2]; m.gmfp0[nge - 1] = gmfp - m.gmfp1[nge - 1] * gle;
        m.gbr11[nge - 1] = m.gbr11[nge - 2]; m.gbr10[nge - 1] = gbr1 - m.gbr11[nge - 1] * gle;
        m.gbr21[nge - 1] = m.gbr21[nge - 2]; m.gbr20[nge - 1] = gbr2 - m.gbr21[nge - 1] * gle;
        m.cohe1[nge - 1] = m.cohe1[nge - 2]; m.cohe0[nge - 1] = cohe - m.cohe1[nge - 1] * gle;
    }

    // ---- mscati (:2750-2979) ----
    {
        LineReader ms;
        if (!ms.open(d + "msnew.data")) { err = "cannot open msnew.data"; return 2; }
        const size_t N = (size_t)MS_NL * MS_NQ * MS_NU;
        H.ums.assign(N, 0); H.fms.assign(N, 0); H.wms.assign(N, 0); H.ims.assign(N, 0);
        for (int i = 0; i < MS_NL; ++i)
            for (int j = 0; j < MS_NQ; ++j) {
                size_t base = ((size_t)i * MS_NQ + j) * MS_NU;
                auto u = ms.read(MS_NU), f = ms.read(MS_NU), w = ms.read(MS_NU - 1), ii = ms.read(MS_NU - 1);
                if (!ms.ok) { err = "bad msnew.data"; return 2; }
                for (int k = 0; k < MS_NU; ++k) { H.ums[base + k] = u[k]; H.fms[base + k] = f[k]; }
                for (int k = 0; k < MS_NU - 1; ++k) {
                    H.wms[base + k] = w[k];
                    H.fms[base + k] = f[k + 1] / f[k] - 1;
                    H.ims[base + k] = (int)ii[k] - 1;
                }
                H.fms[base + MS_NU - 1] = H.fms[base + MS_NU - 2];
            }
        double llammin = std::log(LAMBMIN_MS), llammax = std::log(LAMBMAX_MS);
        H.dllambi = 1. / ((llammax - llammin) / (MS_NL - 1));
        H.dqmsi = 1. / (QMAX_MS / (MS_NQ - 1));
    }
    // PRESTA-I boundary crossing without a skin depth given: the old PRESTA
    // default minimum step, from the lowest ECUT and blcc, xcc as read from
    // PEGS4 (before the conversion below), in elastic MFPs
    // (src/egsnrc.mortran:2794-2815)
    if (!H.params.exact_bca && H.params.skindepth_for_bca <= 1e-4) {
        double ecutmn = 1e30;
        for (auto &m : H.media) ecutmn = std::min(ecutmn, std::max(H.params.ecut, m.ae));
        double tstbmn = 1e30;
        for (auto &m : H.media) {
            double t = (ecutmn - RM) * (ecutmn + RM) / (ecutmn * ecutmn);
            t = m.blcc * t * (ecutmn / m.xcc) * (ecutmn / m.xcc);
            const double aux = std::log(t);
            tstbmn = std::min(tstbmn, std::log(t / aux));
        }
        H.params.skindepth_for_bca = std::exp(tstbmn);
    }
    for (auto &m : H.media) {
        m.blcc = 1.16699413758864573 * m.blcc;
        m.xcc = m.xcc * m.xcc;
    }
    for (auto &m : H.media) {
        const int neke = m.meke;
        double sigee = 1e-15, sigep = 1e-15, sige_old = -1, sigp_old = -1;
        bool emono = true, pmono = true;
        for (int i = 1; i <= neke; ++i) {
            double ei = std::exp((i - m.eke0) / m.eke1), eil = std::log(ei);
            int l = i - 1;
            double ded = m.ededx1[l] * eil + m.ededx0[l];
            double sig = (m.esig1[l] * eil + m.esig0[l]) / ded;
            if (sig > sigee) sigee = sig;
            if (sig < sige_old) emono = false;
            sige_old = sig;
            ded = m.pdedx1[l] * eil + m.pdedx0[l];
            sig = (m.psig1[l] * eil + m.psig0[l]) / ded;
            if (sig > sigep) sigep = sig;
            if (sig < sigp_old) pmono = false;
            sigp_old = sig;
        }
        m.sig_ismonotone[0] = emono;
        m.sig_ismonotone[1] = pmono;
        m.esig_e = sigee;
        m.psig_e = sigep;

        // range to the first table energy
        m.E_array.assign(neke, 0);
        m.range_ep0.assign(neke, 0);
        m.range_ep1.assign(neke, 0);
        double ei = std::exp((1 - m.eke0) / m.eke1);
        m.E_array[0] = ei;
        m.expeke1 = std::exp(1. / m.eke1) - 1;
        for (int i = 1; i <= neke - 1; ++i) {
            double eip1 = std::exp((i + 1 - m.eke0) / m.eke1);
            m.E_array[i] = eip1;
            double eke = 0.5 * (eip1 + ei), elke = std::log(eke);
            int l = set_interval(elke, m.eke1, m.eke0) - 1;
            double ded = m.pdedx1[l] * elke + m.pdedx0[l];
            double aux = m.pdedx1[i - 1] / ded;
            m.range_ep1[i] = m.range_ep1[i - 1] +
                             (eip1 - ei) / ded * (1 + aux * (1 + 2 * aux) * ((eip1 - ei) / eke) * ((eip1 - ei) / eke) / 24);
            ded = m.ededx1[l] * elke + m.ededx0[l];
            aux = m.ededx1[i - 1] / ded;
            m.range_ep0[i] = m.range_ep0[i - 1] +
                             (eip1 - ei) / ded * (1 + aux * (1 + 2 * aux) * ((eip1 - ei) / eke) * ((eip1 - ei) / eke) / 24);
            ei = eip1;
        }
        // tmxs: largest step allowed by estepe and ximax
        const double ximax = params.ximax, estepe = params.estepe;
        double eil = (1 - m.eke0) / m.eke1;
        ei = std::exp(eil);
        double p2 = ei * (ei + 2 * RM), beta2 = p2 / (p2 + RM * RM);
        double chi_a2 = m.xcc / (4 * p2 * m.blcc);
        double dedx0 = m.ededx1[0] * eil + m.ededx0[0];
        double estepx = 2 * p2 * beta2 * dedx0 / ei / m.xcc / (std::log(1 + 1. / chi_a2) * (1 + chi_a2) - 1);
        estepx *= ximax;
        if (estepx > estepe) estepx = estepe;
        double si = estepx * ei / dedx0;
        for (int i = 1; i <= neke - 1; ++i) {
            double elke = (i + 1 - m.eke0) / m.eke1, eke = std::exp(elke);
            int lelke = i + 1;
            p2 = eke * (eke + 2 * RM);
            beta2 = p2 / (p2 + RM * RM);
            chi_a2 = m.xcc / (4 * p2 * m.blcc);
            double ded = m.ededx1[lelke - 1] * elke + m.ededx0[lelke - 1];
            estepx = 2 * p2 * beta2 * ded / eke / m.xcc / (std::log(1 + 1. / chi_a2) * (1 + chi_a2) - 1);
            estepx *= ximax;
            if (estepx > estepe) estepx = estepe;
            double ekef = (1 - estepx) * eke, sip1;
            int lelkef;
            if (ekef <= m.E_array[0]) {
                sip1 = (m.E_array[0] - ekef) / dedx0;
                ekef = m.E_array[0];
                lelkef = 1;
            } else {
                double elkef = std::log(ekef);
                lelkef = set_interval(elkef, m.eke1, m.eke0);
                int leip1l = lelkef + 1;
                double eip1l = (leip1l - m.eke0) / m.eke1, eip1 = m.E_array[leip1l - 1];
                double aux = (eip1 - ekef) / eip1;
                double elktmp = 0.5 * (elkef + eip1l + 0.25 * aux * aux * (1 + aux * (1 + 0.875 * aux)));
                double ektmp = 0.5 * (ekef + eip1);
                int lt = lelkef - 1;
                double dd = m.ededx1[lt] * elktmp + m.ededx0[lt];
                aux = m.ededx1[lt] / dd;
                sip1 = (eip1 - ekef) / dd * (1 + aux * (1 + 2 * aux) * ((eip1 - ekef) / ektmp) * ((eip1 - ekef) / ektmp) / 24);
            }
            sip1 = sip1 + m.range_ep0[lelke - 1] - m.range_ep0[lelkef];
            m.tmxs1[i - 1] = (sip1 - si) * m.eke1;
            m.tmxs0[i - 1] = sip1 - m.tmxs1[i - 1] * elke;
            si = sip1;
        }
        m.tmxs0[neke - 1] = m.tmxs0[neke - 2];
        m.tmxs1[neke - 1] = m.tmxs1[neke - 2];
    }

    // ---- init_compton (:2442-2594); called before EDGSET with EADL + xcom ----
    {
        LineReader ic;
        if (!ic.open(d + "incoh.data")) { err = "cannot open incoh.data"; return 2; }
        ic.skip(18);
        ComptonShells &S = H.shells;
        int izprev = 0;
        while (!ic.eof()) {
            auto v = ic.read_line();
            if (v.size() < 5) break;
            int iz = (int)v[0], shn = (int)v[1];
            double Jo = v[3] * 137., be = v[4] * 1e-6 / RM;
            double erfJo = 0.82436063535 * (std::erf(0.70710678119 * (1 + 0.3 * Jo)) - 1);
            // EADL: shells renumbered per element, binding energies from the photo edges
            if (iz != izprev) { shn = 1; izprev = iz; }
            else shn = S.shn.back() + 1;
            if (shn <= 30) {
                if (binding[iz][shn] > 0) be = binding[iz][shn] / RM;
                else binding[iz][shn] = be * RM;
            }
            S.iz.push_back(iz); S.shn.push_back(shn); S.ne.push_back((int)v[2]);
            S.Jo.push_back(Jo); S.be.push_back(be); S.erfJo.push_back(erfJo);
        }
        if (S.iz.size() != 1538) { err = "incoh.data: unexpected number of shells"; return 2; }
        for (auto &m : H.media) {
            double pztot = 0;
            m.shell_array.clear();
            m.eno_array.clear();
            for (int i = 0; i < m.nne; ++i) {
                int iz = (int)m.zelem[i];
                for (size_t j = 0; j < S.iz.size(); ++j)
                    if (S.iz[j] == iz) {
                        m.shell_array.push_back((int)j);
                        double aux = m.pz[i] * S.ne[j];
                        m.eno_array.push_back(aux);
                        pztot += aux;
                    }
            }
            int nsh = (int)m.shell_array.size();
            if (nsh == 0 || nsh > MXMDSH) { err = "medium " + m.name + ": bad number of Compton shells"; return 3; }
            m.n_shell = nsh;
            // 1-based alias construction exactly as in init_compton
            std::vector<double> eno(nsh + 1);
            std::vector<int> atb(nsh + 1);
            for (int i = 1; i <= nsh; ++i) { eno[i] = -(m.eno_array[i - 1] / pztot); atb[i] = i; }
            double atav = 1. / nsh;
            for (int i = 1; i <= nsh - 1; ++i) {
                int jh, jl;
                for (jh = 1; jh <= nsh - 1; ++jh)
                    if (eno[jh] < 0 && std::fabs(eno[jh]) > atav) break;
                for (jl = 1; jl <= nsh - 1; ++jl)
                    if (eno[jl] < 0 && std::fabs(eno[jl]) < atav) break;
                double aux = atav - std::fabs(eno[jl]);
                eno[jh] += aux;
                eno[jl] = -eno[jl] / atav + jl;
                atb[jl] = jh;
                if (i == nsh - 1) eno[jh] = 1 + jh;
            }
            for (int i = 1; i <= nsh; ++i) if (eno[i] < 0) eno[i] = 1 + i;
            m.eno_array.assign(eno.begin() + 1, eno.end());
            m.eno_atbin_array.assign(atb.begin() + 1, atb.end());
        }
    }

    // ---- EDGSET (:6312-6425): interaction probabilities and edge fits ----
    {
        LineReader pr, pc;
        if (!pr.open(d + "photo_relax.data") || !pc.open(d + "photo_cs.data")) {
            err = "cannot open photo_relax.data / photo_cs.data";
            return 2;
        }
        pr.skip(100);   // binding energies (unused with EADL relaxation)
        pr.skip(1);
        std::vector<std::vector<double>> iprob(101);
        for (int iz = 1; iz <= 100; ++iz) {
            auto v = pr.read_line();
            if (v.size() < 6) { err = "bad photo_relax.data"; return 2; }
            iprob[iz].assign(v.begin() + 1, v.begin() + 6);
        }
        std::map<int, ElementPhoto> ep;
        for (int iz = 1; iz <= 100; ++iz) {
            auto h = pc.read(2);
            int ne = (int)h[1];
            if (!pc.ok || ne > MXEDGE) { err = "bad photo_cs.data"; return 2; }
            ElementPhoto e;
            e.Z = iz;
            e.edge_number = ne;
            for (int j = 0; j < ne; ++j) {
                auto v = pc.read(5);
                e.edge_a[j] = v[0]; e.edge_b[j] = v[1]; e.edge_c[j] = v[2];
                e.edge_d[j] = v[3]; e.edge_energies[j] = v[4];
            }
            for (int k = 0; k < MXINTER; ++k) e.interaction_prob[k] = iprob[iz][k];
            e.interaction_prob[MXSHELL - 1] = 1.01;
            for (int k = 0; k < MXSHELL; ++k) e.binding[k] = binding[iz][k + 1];
            ep[iz] = e;
        }
        H.max_binding_energy = 0;
        for (auto &m : H.media) {
            m.elem_index.clear();
            for (int i = 0; i < m.nne; ++i) {
                int iz = (int)(m.zelem[i] + 0.5);
                int idx = -1;
                for (size_t k = 0; k < H.elements.size(); ++k)
                    if (H.elements[k].Z == iz) idx = (int)k;
                if (idx < 0) { H.elements.push_back(ep[iz]); idx = (int)H.elements.size() - 1; }
                m.elem_index.push_back(idx);
                H.max_binding_energy = std::max(H.max_binding_energy, binding[iz][1]);
            }
            for (int si : m.shell_array)
                H.max_binding_energy = std::max(H.max_binding_energy, H.shells.be[si] * RM);
        }
    }

    // ---- fix_brems (:2322-2413) ----
    for (auto &m : H.media) {
        m.log_ap = std::log(m.ap);
        double Zt = 0, Zb = 0, Zf = 0;
        for (int i = 0; i < m.nne; ++i) {
            double Zi = m.zelem[i], pi = m.pz[i], fc = fcoulc(Zi), xi = xsif(Zi);
            double aux = pi * Zi * (Zi + xi);
            Zt += aux;
            Zb -= aux * std::log(Zi) / 3;
            Zf += aux * fc;
        }
        double Zv = (Zb - Zf) / Zt, Zg = Zb / Zt;
        double fmax1 = 2 * (20.863 + 4 * Zg) - 2 * (20.029 + 4 * Zg) / 3;
        double fmax2 = 2 * (20.863 + 4 * Zv) - 2 * (20.029 + 4 * Zv) / 3;
        double (*dl)[8] = m.dl;   // dl[k][l]: k = dl1..dl6, l = 0..7
        auto set = [&](int l, double a1, double a2, double a3, double a4, double a5, double a6) {
            dl[0][l] = a1; dl[1][l] = a2; dl[2][l] = a3; dl[3][l] = a4; dl[4][l] = a5; dl[5][l] = a6;
        };
        set(0, (20.863 + 4 * Zg) / fmax1, -3.242 / fmax1, 0.625 / fmax1, (21.12 + 4 * Zg) / fmax1, -4.184 / fmax1, 0.952);
        set(1, (20.029 + 4 * Zg) / fmax1, -1.93 / fmax1, -0.086 / fmax1, (21.12 + 4 * Zg) / fmax1, -4.184 / fmax1, 0.952);
        set(2, (20.863 + 4 * Zv) / fmax2, -3.242 / fmax2, 0.625 / fmax2, (21.12 + 4 * Zv) / fmax2, -4.184 / fmax2, 0.952);
        set(3, (20.029 + 4 * Zv) / fmax2, -1.93 / fmax2, -0.086 / fmax2, (21.12 + 4 * Zv) / fmax2, -4.184 / fmax2, 0.952);
        set(4, 3 * (20.863 + 4 * Zg) - (20.029 + 4 * Zg), 3 * (-3.242) - (-1.930), 3 * 0.625 - (-0.086),
            2 * 21.12 + 8 * Zg, 2 * (-4.184), 0.952);
        set(5, 3 * (20.863 + 4 * Zg) + (20.029 + 4 * Zg), 3 * (-3.242) + (-1.930), 3 * 0.625 + (-0.086),
            4 * 21.12 + 16 * Zg, 4 * (-4.184), 0.952);
        set(6, 3 * (20.863 + 4 * Zv) - (20.029 + 4 * Zv), 3 * (-3.242) - (-1.930), 3 * 0.625 - (-0.086),
            2 * 21.12 + 8 * Zv, 2 * (-4.184), 0.952);
        set(7, 3 * (20.863 + 4 * Zv) + (20.029 + 4 * Zv), 3 * (-3.242) + (-1.930), 3 * 0.625 + (-0.086),
            4 * 21.12 + 16 * Zv, 4 * (-4.184), 0.952);
        m.bpar[1] = dl[0][6] / (3 * dl[0][7] + dl[0][6]);
        m.bpar[0] = 12 * dl[0][7] / (3 * dl[0][7] + dl[0][6]);
    }
    return 0;
}

}  // namespace egs
