// ORACLE -- test infrastructure only.  A C harness around the reference's own
// egs++ classes for the voxel path, compiled from the reference's sources
// where they lie (oracle/Makefile, target `ref`, into oracle/_ref/, which is
// not committed).  The tests use it to pin the engine's and the restatement's
// geometry and source against the reference's code itself:
//   EGS_XYZGeometry isWhere / howfar / hownear / howfarFromOut
//     (egs++/geometry/egs_nd_geometry/egs_nd_geometry.h:769-1379), built on
//     EGS_PlanesX/Y/Z (egs++/geometry/egs_planes/egs_planes.h:200-300);
//   EGS_ParallelBeam (egs++/sources/egs_parallel_beam/egs_parallel_beam.h:150)
//     over an EGS_RectangleShape (egs++/shapes/egs_rectangle/egs_rectangle.h:87)
//     with the spectrum that EGS_BaseSpectrum::createSpectrum builds from an
//     egs++ input block (egs++/egs_spectra.cpp:466-800), sampled with the
//     reference's default generator (RANMAR, egs++/egs_rndm.cpp);
//   EGS_Application::simulateSingleShower's entry of a source particle into
//     the geometry (egs++/egs_application.cpp:919-945).
// Only this file is ours; the classes are the reference's.  Nothing here is
// shipped or used by the product path.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "egs_application.h"
#include "egs_base_source.h"
#include "egs_input.h"
#include "egs_rndm.h"
#include "egs_vector.h"
#include "geometry/egs_nd_geometry/egs_nd_geometry.h"
#include "geometry/egs_planes/egs_planes.h"
#include "shapes/egs_rectangle/egs_rectangle.h"
#include "sources/egs_parallel_beam/egs_parallel_beam.h"

// The classes report through the active application when there is one;
// this harness runs without an application, so they print to stderr.
EGS_Application *EGS_Application::activeApplication() { return nullptr; }

extern "C" {

// An XYZ geometry from plane positions (nx+1, ny+1, nz+1 values, cm).
void *egsref_xyz_new(int nx, int ny, int nz, const double *xb, const double *yb, const double *zb) {
    // as EGS_XYZGeometry's own factory builds it (egs_nd_geometry.cpp:721-724),
    // with names of our own: egs++ refuses two live geometries of one name
    static long long serial = 0;
    const std::string tag = std::to_string(++serial);
    EGS_PlanesX *px = new EGS_PlanesX(nx + 1, xb, "ref_x" + tag, EGS_XProjector("x-planes"));
    EGS_PlanesY *py = new EGS_PlanesY(ny + 1, yb, "ref_y" + tag, EGS_YProjector("y-planes"));
    EGS_PlanesZ *pz = new EGS_PlanesZ(nz + 1, zb, "ref_z" + tag, EGS_ZProjector("z-planes"));
    return new EGS_XYZGeometry(px, py, pz, "ref_xyz" + tag);
}

void egsref_xyz_free(void *g) { delete (EGS_XYZGeometry *)g; }

double egsref_boundary_tolerance(void *g) { return ((EGS_XYZGeometry *)g)->getBoundaryTolerance(); }

// isWhere of n points (x[3n]).
void egsref_xyz_iswhere(void *g, long long n, const double *x, int *ireg) {
    EGS_XYZGeometry *G = (EGS_XYZGeometry *)g;
    for (long long i = 0; i < n; ++i) ireg[i] = G->isWhere(EGS_Vector(x[3 * i], x[3 * i + 1], x[3 * i + 2]));
}

// howfar of n queries: region ireg[i] (< 0: from outside), position x, unit
// direction u, step t[i] on entry; returns the new region in inew[i] and
// the (possibly shortened) step in t[i].
void egsref_xyz_howfar(void *g, long long n, const int *ireg, const double *x, const double *u, double *t,
                       int *inew) {
    EGS_XYZGeometry *G = (EGS_XYZGeometry *)g;
    for (long long i = 0; i < n; ++i) {
        EGS_Float tt = t[i];
        inew[i] = G->howfar(ireg[i], EGS_Vector(x[3 * i], x[3 * i + 1], x[3 * i + 2]),
                            EGS_Vector(u[3 * i], u[3 * i + 1], u[3 * i + 2]), tt);
        t[i] = tt;
    }
}

// hownear of n points in regions ireg[i] >= 0.
void egsref_xyz_hownear(void *g, long long n, const int *ireg, const double *x, double *tperp) {
    EGS_XYZGeometry *G = (EGS_XYZGeometry *)g;
    for (long long i = 0; i < n; ++i) tperp[i] = G->hownear(ireg[i], EGS_Vector(x[3 * i], x[3 * i + 1], x[3 * i + 2]));
}

// Source particles of an egs++ parallel beam with a rectangle shape
// {xmin, xmax, ymin, ymax} in the plane z = z0, direction dir, charge q and
// the spectrum of the egs++ input text `spectrum` (a ":start spectrum:"
// block), each entered into geometry g (when g is not NULL) as
// simulateSingleShower does: isWhere, then howfar from outside with
// t = veryFar and x += u t.  out[9 i ...] = {q, E (kinetic), x, y, z, u, v,
// w, region}.  Returns the number of particles, or -1 on an input error.
long long egsref_parallel_beam(const char *spectrum, int q, const double *rect, double z0, const double *dir,
                               void *g, long long n, int seed, double *out) {
    EGS_Input inp;
    std::string text(spectrum);
    if (inp.setContentFromString(text)) return -1;
    EGS_BaseSpectrum *spec = EGS_BaseSpectrum::createSpectrum(&inp);
    if (!spec) return -1;
    EGS_RectangleShape *shape = new EGS_RectangleShape(rect[0], rect[1], rect[2], rect[3]);
    shape->setTransformation(new EGS_AffineTransform(EGS_Vector(0, 0, z0)));
    EGS_ParallelBeam src(q, spec, shape, "ref_beam");
    // EGS_ParallelBeam's direction comes from its input; this constructor
    // keeps +z, so other directions are rejected rather than ignored
    if (dir && (dir[0] != 0 || dir[1] != 0 || dir[2] != 1)) return -1;
    EGS_RandomGenerator *rng = EGS_RandomGenerator::defaultRNG(seed);
    EGS_XYZGeometry *G = (EGS_XYZGeometry *)g;
    for (long long i = 0; i < n; ++i) {
        int qq;
        int latch;
        EGS_Float E, wt;
        EGS_Vector x, u;
        src.getNextParticle(rng, qq, latch, E, wt, x, u);
        int ireg = -1;
        if (G) {
            ireg = G->isWhere(x);
            if (ireg < 0) {
                EGS_Float t = veryFar;
                ireg = G->howfar(ireg, x, u, t);
                if (ireg >= 0) x += u * t;
            }
        }
        double *o = out + 9 * i;
        o[0] = qq; o[1] = E; o[2] = x.x; o[3] = x.y; o[4] = x.z; o[5] = u.x; o[6] = u.y; o[7] = u.z; o[8] = ireg;
    }
    delete rng;
    return n;
}

}  // extern "C"
