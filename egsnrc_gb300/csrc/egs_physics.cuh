// Device interaction samplers.  Each routine restates one EGSnrc routine
// (paths relative to HEN_HOUSE) and draws its random numbers from the
// interacting particle's own Philox stream, in the reference's order.
#pragma once
#include "egs_device.cuh"

namespace egsgpu {

template <class Real>
struct Particle {
    Real x, y, z, u, v, w, E, wt;
    int ir, iq;
    int pb;       // phantom of a multi-phantom run (derived from ir; not stored in queues)
    Rng rng;
};

template <class Real>
struct Azim { Real c, s; };

// $SELECT-AZIMUTHAL-ANGLE (src/egsnrc.macros:2491-2509)
// out of line: see Rng::u (egs_device.cuh)
template <class Real>
__device__ __noinline__ Azim<Real> azimuth(Rng &r, int &err) {
    Real xphi, xphi2, yphi, yphi2, rho2;
    int it = 0;
    do {
        float2 q = urand2(r);
        xphi = (Real)q.x; xphi = 2 * xphi - 1; xphi2 = xphi * xphi;
        yphi = (Real)q.y; yphi2 = yphi * yphi;
        rho2 = xphi2 + yphi2;
        if (++it > LOOP_CAP) { err = 1; break; }
    } while (rho2 > 1);
    rho2 = 1 / rho2;
    return {(xphi2 - yphi2) * rho2, 2 * xphi * yphi * rho2};
}

// UPHI :ADJUST: (src/egsnrc.mortran:6820-6838)
template <class Real>
__device__ inline void rotate(Real a, Real b, Real c, Real sinthe, Real costhe, Azim<Real> az, Real &u,
                              Real &v, Real &w) {
    Real sinps2 = a * a + b * b;
    if (sinps2 < (Real)1e-20) {
        u = sinthe * az.c; v = sinthe * az.s; w = c * costhe;
    } else {
        Real sinpsi = dsqrt(sinps2), us = sinthe * az.c, vs = sinthe * az.s;
        Real sindel = b / sinpsi, cosdel = a / sinpsi;
        u = c * cosdel * us - sindel * vs + a * costhe;
        v = c * sindel * us + cosdel * vs + b * costhe;
        w = -sinpsi * us + c * costhe;
    }
}

// ------------------------------------------------------------ Rayleigh ----
// egs_rayleigh_sampling (src/egsnrc.mortran:8559-8590)
template <class Real>
__device__ inline void rayleigh(const Tables<Real> &T, int med, Real E, Real gle, int lgle, Rng &r,
                                Real &costhe, Real &sinthe, int &err) {
    const Real hc_i = (Real)80.65506856998, twice_hc2 = (Real)0.000307444456, dwi = (Real)(NRAY - 1);
    const Real *pm = T.pmax + ((size_t)med * MXGE + (lgle - 1)) * 2;
    const Real *xg = T.ray + (size_t)med * 4 * NRAY, *fc = xg + NRAY, *ba = fc + NRAY, *ca = ba + NRAY;
    const int *ia = T.ray_i + (size_t)med * NRAY;
    Real pmax = pm[1] * gle + pm[0], xmax = hc_i * E, xv, csq, rn1;
    int it = 0;
    do {
        rn1 = urand<Real>(r);
        do {
            Real r0 = urand<Real>(r) * pmax;
            int ibin = 1 + (int)(r0 * dwi);
            int ib = ia[ibin - 1];
            if (ia[ibin] > ib) {
                while (!(r0 < fc[ib]) && ib < NRAY - 1) ++ib;
            }
            r0 = (r0 - fc[ib - 1]) * ca[ib - 1];
            xv = xg[ib - 1] * dexp(dlog(1 + r0) * ba[ib - 1]);
            if (++it > LOOP_CAP) { err = 1; break; }
        } while (!(xv < xmax));
        xv = xv / E;
        costhe = 1 - twice_hc2 * xv * xv;
        csq = costhe * costhe;
        if (it > LOOP_CAP) break;
    } while (!(2 * rn1 < 1 + csq));
    sinthe = dsqrt(dmax((Real)0, 1 - csq));
}

// ------------------------------------------------------------- Compton ----
// COMPT with bound-electron corrections, ibcmp = 3 (src/egsnrc.mortran:528-805).
// The photon is updated in place; the electron direction/energy returned.
// Returns the binding energy deposited locally (relaxation products are all
// below the transport cut-offs, which the host checks).
template <class Real>
__device__ inline Real compton(const Tables<Real> &T, const MedScalars<Real> &M, Particle<Real> &p,
                               Real &eu, Real &ev, Real &ew, Real &eE, int &err) {
    Rng &r = p.rng;
    const Real rm = (Real)RM;
    Real peig = p.E, ko = peig / rm, broi = 1 + 2 * ko;
    bool first_time = true;
    Real Uj = 0, Jo = 0, erfJo = 0, br = 0, temp = 0, sinthe = 0, costhe = 0;
    Real alph1 = 0, alpha = 0, bro = 0, broi2 = 0, bro1 = 0, rejmax = 0;
    Real Fmax = 1, fpz = 1, af = 0, qc = 0, qc2 = 0, br2 = 0;
    int guard = 0;
    while (true) {   // :resample-compton:
        if (++guard > LOOP_CAP) { err = 1; break; }
        Real r17 = urand<Real>(r);
        r17 = 1 + r17 * M.n_shell;
        int i = (int)r17;
        const Real *sh = T.shell + (size_t)(M.shell_off + i - 1) * 4;
        if (r17 > sh[0]) {
            i = T.shell_at[M.shell_off + i - 1];
            sh = T.shell + (size_t)(M.shell_off + i - 1) * 4;
        }
        Uj = sh[1];
        if (ko <= Uj) continue;
        Jo = sh[2];
        erfJo = sh[3];
        int g2 = 0;
        do {   // :RESAMPLE: Klein-Nishina
            if (ko > 2) {
                if (first_time) {
                    broi2 = broi * broi; alph1 = dlog(broi); bro = 1 / broi;
                    Real alph2 = ko * (broi + 1) * bro * bro;
                    alpha = alph1 + alph2;
                }
                Real r15, r16, r19, aux, rejf3;
                int it = 0;
                do {
                    r15 = urand<Real>(r); r16 = urand<Real>(r);
                    if (r15 * alpha < alph1) br = dexp(alph1 * r16) * bro;
                    else br = dsqrt(r16 * broi2 + (1 - r16)) * bro;
                    temp = (1 - br) / (ko * br);
                    sinthe = dmax((Real)0, temp * (2 - temp));
                    aux = 1 + br * br;
                    rejf3 = aux - br * sinthe;
                    r19 = urand<Real>(r);
                    if (++it > LOOP_CAP) { err = 1; break; }
                } while (!(r19 * aux <= rejf3));
            } else {
                if (first_time) { bro = 1 / broi; bro1 = 1 - bro; rejmax = broi + bro; }
                Real r15, r16, rejf3;
                int it = 0;
                do {
                    r15 = urand<Real>(r); r16 = urand<Real>(r);
                    br = bro + bro1 * r15;
                    temp = (1 - br) / (ko * br);
                    sinthe = dmax((Real)0, temp * (2 - temp));
                    rejf3 = 1 + br * br - br * sinthe;
                    if (++it > LOOP_CAP) { err = 1; break; }
                } while (!(r16 * br * rejmax <= rejf3));
            }
            first_time = false;
            if (++g2 > LOOP_CAP) { err = 1; break; }
        } while (br < bro || br > 1);
        costhe = 1 - temp;
        br2 = br * br;
        Real aux = ko * (ko - Uj) * temp, aux1 = 2 * aux + Uj * Uj;
        Real pzmax = aux - Uj;
        if (pzmax < 0 && pzmax * pzmax >= aux1) continue;
        pzmax = pzmax / dsqrt(aux1);
        qc2 = 1 + br * br - 2 * br * costhe;
        qc = dsqrt(qc2);
        if (pzmax > 1) { af = 0; Fmax = 1; fpz = 1; break; }
        Real aux3 = 1 + 2 * Jo * dabs(pzmax), aux4 = (Real)0.5 * (1 - aux3 * aux3);
        fpz = (Real)0.5 * dexp(aux4);
        af = qc * (1 + br * (br - costhe) / qc2);
        if (af < 0) {
            if (pzmax > 0) fpz = 1 - fpz;
            Real eta = urand<Real>(r);
            if (eta > fpz) continue;
            af = 0; Fmax = 1;
            break;
        }
        Real fpz1;
        if (pzmax < (Real)-0.15) { Fmax = 1 - af * (Real)0.15; fpz1 = fpz * Fmax * Jo; }
        else if (pzmax < (Real)0.15) {
            Fmax = 1 + af * pzmax;
            aux3 = 1 / (1 + (Real)0.33267252734 * aux3);
            aux4 = fpz * aux3 * ((Real)0.3480242 + aux3 * ((Real)-0.0958798 + aux3 * (Real)0.7478556)) + erfJo;
            if (pzmax > 0) { fpz1 = (1 - Fmax * fpz) * Jo - (Real)0.62665706866 * af * aux4; fpz = 1 - fpz; }
            else fpz1 = Fmax * fpz * Jo - (Real)0.62665706866 * af * aux4;
        } else { Fmax = 1 + af * (Real)0.15; fpz1 = (1 - Fmax * fpz) * Jo; fpz = 1 - fpz; }
        Real eta = urand<Real>(r);
        if (eta * Jo > fpz1) continue;
        break;
    }
    // :RETRY-PZ:
    Real pz;
    int it = 0;
    while (true) {
        Real r18 = urand<Real>(r) * fpz;
        if (r18 < (Real)0.5) {
            r18 = dmax((Real)1e-30, 2 * r18);
            pz = (Real)0.5 * (1 - dsqrt(1 - 2 * dlog(r18))) / Jo;
        } else {
            r18 = 2 * (1 - r18);
            pz = (Real)0.5 * (dsqrt(1 - 2 * dlog(r18)) - 1) / Jo;
        }
        if (++it > LOOP_CAP) { err = 1; break; }
        if (dabs(pz) > 1) continue;
        if (pz < (Real)0.15) {
            Real frej = (pz < (Real)-0.15) ? 1 - af * (Real)0.15 : 1 + af * pz;
            Real eta = urand<Real>(r);
            if (eta * Fmax > frej) continue;
        }
        break;
    }
    Real pz2 = pz * pz;
    if (dabs(pz) < (Real)0.01) br = br * (1 + pz * (qc + (br2 - costhe) * pz));
    else {
        Real a1 = 1 - pz2 * br * costhe, a2 = 1 - pz2 * br2, a3 = qc2 - br2 * pz2 * sinthe;
        if (a3 > (Real)1e-10) br = br / a2 * (a1 + pz * dsqrt(a3));
    }
    Uj = Uj * rm;
    Real pesg = br * peig, pese = peig - pesg - Uj + rm;
    sinthe = dsqrt(sinthe);
    Azim<Real> az = azimuth<Real>(r, err);
    Real a = p.u, b = p.v, c = p.w;
    rotate(a, b, c, sinthe, costhe, az, p.u, p.v, p.w);
    p.E = pesg;
    Real aux = 1 + br * br - 2 * br * costhe, ce, se;
    if (aux > (Real)1e-8) {
        ce = (1 - br * costhe) / dsqrt(aux);
        se = (1 - ce) * (1 + ce);
        se = (se > 0) ? -dsqrt(se) : (Real)0;
    } else { ce = 0; se = -1; }
    rotate(a, b, c, se, ce, az, eu, ev, ew);
    eE = pese;
    return Uj;
}

// --------------------------------------------------------------- PHOTO ----
// PHOTO with EADL edges (src/egsnrc.mortran:5050-5195) and the Sauter
// photo-electron direction (src/egsnrc.macros:1916-1955). Converts p into the
// photo-electron; returns the vacancy energy deposited locally.
template <class Real>
__device__ inline Real photo(const Tables<Real> &T, const MedScalars<Real> &M, Particle<Real> &p, Real gle,
                             int &err) {
    Rng &r = p.rng;
    const Real rm = (Real)RM;
    Real peig = p.E, e_vac = 0;
    const Real *el;
    if (M.nne == 1) {
        el = T.elem + (size_t)M.elem_off * 96;
    } else {
        Real aux = peig * peig, aux1 = aux * peig;
        aux = aux * dsqrt(peig);
        Real probs[MAXNE], sigtot = 0;
        for (int k = 0; k < M.nne; ++k) {
            const Real *e = T.elem + (size_t)(M.elem_off + k) * 96;
            int ne = (int)e[95];
            Real sigma;
            if (peig > e[64]) {
                sigma = (e[0] + e[16] / peig + e[32] / aux + e[48] / aux1) / peig;
            } else {
                int j;
                for (j = 1; j < ne; ++j) if (peig >= e[64 + j]) break;
                if (j >= ne) j = ne - 1;
                sigma = e[j] + gle * (e[16 + j] + gle * (e[32 + j] + gle * e[48 + j]));
                sigma = dexp(sigma);
            }
            sigma *= (Real)M.pz[k];
            sigtot += sigma;
            probs[k] = sigma;
        }
        Real br = urand<Real>(r) * sigtot;
        int k;
        for (k = 0; k < M.nne; ++k) { br -= probs[k]; if (br <= 0) break; }
        if (k >= M.nne) k = M.nne - 1;
        el = T.elem + (size_t)(M.elem_off + k) * 96;
    }
    const Real *bind = el + 80, *iprob = el + 86;
    Real enew;
    if (peig <= bind[5]) {
        enew = peig + rm;
    } else {
        Real br = urand<Real>(r);
        int k;
        for (k = 0; k < 5; ++k) {
            if (peig > bind[k]) {
                if (br < iprob[k]) break;
                br = (br - iprob[k]) / (1 - iprob[k]);
            }
        }
        if (k > 3) enew = peig + rm;
        else { e_vac = bind[k]; enew = peig - e_vac + rm; }
    }
    p.iq = -1;
    p.E = enew;
    if (p.E > T.ecut) {
        Real eelec = p.E, beta = dsqrt((eelec - rm) * (eelec + rm)) / eelec, gamma = eelec / rm;
        Real alpha = (Real)0.5 * gamma - (Real)0.5 + 1 / gamma, ratio = beta / alpha, costhe, sinth2, xi;
        int it = 0;
        while (true) {
            Real rn = urand<Real>(r);
            rn = 2 * rn - 1;
            if (ratio <= (Real)0.2) {
                Real fk = rn + (Real)0.5 * ratio * (1 - rn) * (1 + rn);
                if (gamma < 100) costhe = (beta + fk) / (1 + beta * fk);
                else if (fk > 0) costhe = 1 - (1 - fk) * (gamma - 3) / (2 * (1 + fk) * (gamma - 1) * (gamma - 1) * (gamma - 1));
                else costhe = (beta + fk) / (1 + beta * fk);
                xi = (1 + beta * fk) * gamma * gamma;
            } else {
                xi = gamma * gamma * (1 + alpha * (dsqrt(1 + ratio * (2 * rn + ratio)) - 1));
                costhe = (1 - 1 / xi) / beta;
            }
            sinth2 = dmax((Real)0, (1 - costhe) * (1 + costhe));
            Real rn2 = urand<Real>(r);
            if (!(rn2 > (Real)0.5 * (1 + gamma) * sinth2 * xi / gamma)) break;
            if (++it > LOOP_CAP) { err = 1; break; }
        }
        Real sinthe = dsqrt(sinth2);
        Azim<Real> az = azimuth<Real>(r, err);
        Real a = p.u, b = p.v, c = p.w;
        rotate(a, b, c, sinthe, costhe, az, p.u, p.v, p.w);
    }
    return e_vac;
}

// ---------------------------------------------------------------- PAIR ----
// PAIR (src/egsnrc.mortran:4518-4715) with $SET-PAIR-ANGLE iprdst = 1
// (src/egsnrc.macros:2070-2125) and the low-energy uniform split (:2179-2185).
template <class Real>
__device__ inline void pair(const MedScalars<Real> &M, Particle<Real> &p, Real &E2, int &iq2, Real &u2, Real &v2,
                            Real &w2, int &err) {
    Rng &r = p.rng;
    const Real rm = (Real)RM, rmt2 = (Real)(2 * RM);
    Real peig = p.E, eig = peig, pese1, pese2;
    int iq1;
    if (eig <= (Real)2.1) {
        Real r30 = urand<Real>(r), r34 = urand<Real>(r);
        pese2 = rm + (Real)0.5 * r30 * (peig - 2 * rm);
        pese1 = peig - pese2;
        if (r34 < (Real)0.5) { iq1 = -1; iq2 = 1; } else { iq1 = 1; iq2 = -1; }
    } else {
        int l;
        Real Amax, Bmax, aux1;
        if (eig < 50) {
            l = 4;
            Real delta = 4 * M.delcm / eig;
            if (delta < 1) {
                Amax = M.dl[0][l] + delta * (M.dl[1][l] + delta * M.dl[2][l]);
                Bmax = M.dl[0][l + 1] + delta * (M.dl[1][l + 1] + delta * M.dl[2][l + 1]);
            } else {
                Real aux2 = dlog(delta + M.dl[5][l]);
                Amax = M.dl[3][l] + M.dl[4][l] * aux2;
                Bmax = M.dl[3][l + 1] + M.dl[4][l + 1] * aux2;
            }
            aux1 = 1 - rmt2 / eig;
            aux1 = aux1 * aux1;
            aux1 = aux1 * Amax / 3;
            aux1 = aux1 / (Bmax + aux1);
        } else {
            l = 6;
            Amax = M.dl[0][l]; Bmax = M.dl[0][l + 1];
            aux1 = M.bpar[1] * (1 - M.bpar[0] * rm / eig);
        }
        Real del0 = eig * M.delcm, Eavail = eig - rmt2, br, Eminus, rejmax, rejf, r34;
        int it = 0;
        do {
            Real r30 = urand<Real>(r), r31 = urand<Real>(r);
            r34 = urand<Real>(r);
            int lr;
            if (r30 > aux1) { br = (Real)0.5 * r31; rejmax = Bmax; lr = l + 1; }
            else {
                Real r32 = urand<Real>(r), r33 = urand<Real>(r);
                br = (Real)0.5 * (1 - dmax(r31, dmax(r32, r33)));
                rejmax = Amax; lr = l;
            }
            Eminus = br * Eavail + rm;
            Real Eplus = eig - Eminus, delta = del0 / (Eminus * Eplus);
            if (delta < 1) rejf = M.dl[0][lr] + delta * (M.dl[1][lr] + delta * M.dl[2][lr]);
            else rejf = M.dl[3][lr] + M.dl[4][lr] * dlog(delta + M.dl[5][lr]);
            if (++it > LOOP_CAP) { err = 1; break; }
        } while (!(r34 * rejmax <= rejf));
        pese2 = Eminus;
        pese1 = peig - pese2;
        r34 = urand<Real>(r);
        if (r34 < (Real)0.5) { iq1 = -1; iq2 = 1; } else { iq1 = 1; iq2 = -1; }
    }
    Real a = p.u, b = p.v, c = p.w;
    Azim<Real> az{0, 0};
    Real ese = pese1, pse = dsqrt(dmax((Real)0, (ese - rm) * (ese + rm)));
    Real costhe = urand<Real>(r);
    costhe = 1 - 2 * costhe;
    Real sinthe = rm * dsqrt((1 - costhe) * (1 + costhe)) / (pse * costhe + ese);
    costhe = (ese * costhe + pse) / (pse * costhe + ese);
    az = azimuth<Real>(r, err);
    Real u1, v1, w1;
    rotate(a, b, c, sinthe, costhe, az, u1, v1, w1);
    ese = pese2;
    pse = dsqrt(dmax((Real)0, (ese - rm) * (ese + rm)));
    costhe = urand<Real>(r);
    costhe = 1 - 2 * costhe;
    sinthe = -(rm * dsqrt((1 - costhe) * (1 + costhe)) / (pse * costhe + ese));
    costhe = (ese * costhe + pse) / (pse * costhe + ese);
    rotate(a, b, c, sinthe, costhe, az, u2, v2, w2);
    p.E = pese1; p.iq = iq1; p.u = u1; p.v = v1; p.w = w1;
    E2 = pese2;
}

// ------------------------------------------------------ multiple scatter ----
template <class Real>
struct MsState { bool find_index; int i, j; Real omega2; };

// mscat, spin effects off (src/egsnrc.mortran:2984-3136)
template <class Real>
__device__ inline void mscat(const Tables<Real> &T, Rng &r, Real lambda, Real chia2, Real q1, MsState<Real> &st,
                             Real &cost, Real &sint, int &err) {
    if (lambda <= (Real)13.8) {
        Real sprob = urand<Real>(r), explambda = dexp(-lambda);
        if (sprob < explambda) { cost = 1; sint = 0; return; }
        Real wsum = (1 + lambda) * explambda;
        if (sprob < wsum) {
            Real xi = urand<Real>(r);
            xi = 2 * chia2 * xi / (1 - xi + chia2);
            cost = 1 - xi;
            sint = dsqrt(xi * (2 - xi));
            return;
        }
        if (lambda <= 1) {
            Real wprob = explambda;
            wsum = explambda;
            cost = 1; sint = 0;
            int icount = 0;
            do {
                ++icount;
                if (icount > 20) break;
                wprob = wprob * lambda / icount;
                wsum += wprob;
                Real xi = urand<Real>(r);
                xi = 2 * chia2 * xi / (1 - xi + chia2);
                Real cosz = 1 - xi, sinz = xi * (2 - xi);
                if (sinz > (Real)1e-20) {
                    sinz = dsqrt(sinz);
                    xi = urand<Real>(r);
                    Real phi = xi * (Real)6.2831853;
                    cost = cost * cosz - sint * sinz * dcos(phi);
                    sint = dsqrt(dmax((Real)0, (1 - cost) * (1 + cost)));
                }
            } while (!(wsum > sprob));
            return;
        }
    }
    if (lambda <= (Real)1e5) {
        if (st.find_index) {
            Real llmbda = dlog(lambda);
            Real ai = llmbda * T.dllambi;
            int i = (int)ai;
            ai -= i;
            const bool drawj = !(q1 < (Real)1e-3) && q1 < (Real)0.5;
            float2 qij;
            if (drawj) qij = urand2(r); else qij = make_float2(r.u(), 0.f);
            Real xi = (Real)qij.x;
            if (xi < ai) ++i;
            i = min(max(i, 0), MS_NL - 1);
            int j;
            if (q1 < (Real)1e-3) j = 0;
            else if (q1 < (Real)0.5) {
                Real aj = q1 * T.dqmsi;
                j = (int)aj;
                aj -= j;
                xi = (Real)qij.y;
                if (xi < aj) ++j;
            } else j = MS_NQ - 1;
            Real om;
            if (llmbda < (Real)2.2299)
                om = chia2 * (lambda + 4) * ((Real)1.347006 + llmbda * ((Real)0.209364 - llmbda * ((Real)0.45525 - llmbda * ((Real)0.50142 - (Real)0.081234 * llmbda))));
            else
                om = chia2 * (lambda + 4) * ((Real)-2.77164 + llmbda * ((Real)2.94874 - llmbda * ((Real)0.1535754 - llmbda * (Real)0.00552888)));
            st.omega2 = om;
            st.i = i; st.j = j;
            st.find_index = false;
        }
        const float2 qku = urand2(r);
        Real xi = (Real)qku.x;
        Real ak = xi * (MS_NU - 1);
        int k = (int)ak;
        ak -= k;
        int base = (st.i * MS_NQ + st.j) * MS_NU;
        if (ak > T.ms[(base + k) * 3 + 2]) k = T.ms_i[base + k];
        k = min(max(k, 0), MS_NU - 2);
        Real a = T.ms[(base + k) * 3 + 1], u = T.ms[(base + k) * 3], du = T.ms[(base + k + 1) * 3] - u;
        xi = (Real)qku.y;
        if (dabs(a) < (Real)0.2) {
            Real x1 = (Real)0.5 * (1 - xi) * a;
            u = u + xi * du * (1 + x1 * (1 - xi * a));
        } else u = u - du / a * (1 - dsqrt(1 + xi * a * (2 + a)));
        Real om = st.omega2;
        xi = om * u / (1 + (Real)0.5 * om - u);
        if (xi > (Real)1.99999) xi = (Real)1.99999;
        cost = 1 - xi;
        sint = dsqrt(xi * (2 - xi));
        return;
    }
    err = 1;
    cost = 1; sint = 0;
}

// msdist_pII, spin effects off (src/egsnrc.mortran:4050-4294)
template <class Real>
__device__ inline void msdist_pII(const Tables<Real> &T, const MedScalars<Real> &M, Particle<Real> &p, Real e0,
                                  Real eloss, Real tustep, Real rhof, Real &us, Real &vs, Real &ws, Real &xf,
                                  Real &yf, Real &zf, int &err) {
    const Real rm = (Real)RM;
    Real blccc = M.blcc, xcccc = M.xcc;
    Real e = e0 - (Real)0.5 * eloss, tau = e / rm, tau2 = tau * tau, epsilon = eloss / e0, epsilonp = eloss / e;
    e = e * (1 - epsilonp * epsilonp * (6 + 10 * tau + 5 * tau2) / (24 * tau2 + 72 * tau + 48));
    Real p2 = e * (e + 2 * rm), beta2 = p2 / (p2 + rm * rm);
    Real chia2 = xcccc / (4 * p2 * blccc);
    Real lambda = (Real)0.5 * tustep * rhof * blccc / beta2;
    Real tt = epsilonp / ((tau + 1) * (tau + 2));
    Real temp2 = (Real)0.166666 * (4 + tau * (6 + tau * (7 + tau * (4 + tau)))) * tt * tt;
    lambda = lambda * (1 - temp2);
    lambda = lambda / (1 + chia2);
    Real chilog = dlog(1 + 1 / chia2);
    Real q1 = 2 * chia2 * (chilog * (1 + chia2) - 1);
    Real gamma = 6 * chia2 * (1 + chia2) * (chilog * (1 + 2 * chia2) - 2) / q1;
    Real xi = q1 * lambda;
    MsState<Real> st;
    st.find_index = true; st.i = 0; st.j = 0; st.omega2 = 0;
    // the two half-step deflections share one copy of the sampling code
    // (same random-number order: mscat, azimuth, mscat, azimuth)
    Real w1 = 0, sint1 = 0, w2 = 0, sint2 = 0;
    Azim<Real> a1{0, 0}, a2{0, 0};
#pragma unroll 1
    for (int half = 0; half < 2; ++half) {
        Real wh, sh;
        mscat(T, p.rng, lambda, chia2, xi, st, wh, sh, err);
        Azim<Real> ah = azimuth<Real>(p.rng, err);
        if (half == 0) { w1 = wh; sint1 = sh; a1 = ah; } else { w2 = wh; sint2 = sh; a2 = ah; }
    }
    Real cphi1 = a1.c, sphi1 = a1.s, cphi2 = a2.c, sphi2 = a2.s;
    Real u2 = sint2 * cphi2, v2 = sint2 * sphi2, u2p = w1 * u2 + sint1 * w2;
    us = u2p * cphi1 - v2 * sphi1;
    vs = u2p * sphi1 + v2 * cphi1;
    ws = w1 * w2 - sint1 * u2;
    xi = 2 * xi;
    Real eta = urand<Real>(p.rng);
    eta = dsqrt(eta);
    Real eta1 = (Real)0.5 * (1 - eta);
    Real delta = (Real)0.9082483 - ((Real)0.1020621 - (Real)0.0263747 * gamma) * xi;
    Real temp1 = 2 + tau;
    Real temp = (2 + tau * temp1) / ((tau + 1) * temp1);
    temp = temp - (tau + 1) / ((tau + 2) * (chilog * (1 + chia2) - 1));
    temp = temp * epsilonp;
    temp1 = 1 - temp;
    delta = delta + (Real)0.40824829 * (epsilon * (tau + 1) / ((tau + 2) * (chilog * (1 + chia2) - 1) *
                                                              (chilog * (1 + 2 * chia2) - 2)) - (Real)0.25 * temp * temp);
    Real b = eta * delta, c = eta * (1 - delta);
    Real w1v2 = w1 * v2;
    Real ut = b * sint1 * cphi1 + c * (cphi1 * u2 - sphi1 * w1v2) + eta1 * us * temp1;
    Real vt = b * sint1 * sphi1 + c * (sphi1 * u2 + cphi1 * w1v2) + eta1 * vs * temp1;
    Real wt = eta1 * (1 + temp) + b * w1 + c * w2 + eta1 * ws * temp1;
    Real u0 = p.u, v0 = p.v, w0 = p.w;
    Real sint02 = u0 * u0 + v0 * v0;
    if (sint02 > (Real)1e-20) {
        Real sint0 = dsqrt(sint02), sint0i = 1 / sint0, cphi0 = sint0i * u0, sphi0 = sint0i * v0;
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

}  // namespace egsgpu
