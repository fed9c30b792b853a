// An egs++ application that hands the particle-history loop of the
// egs_ndgeometry XYZ path to libegsgpu: the reference-side binding of this
// library.  It is an EGS_AdvancedApplication (egs++/egs_advanced_application.h)
// whose runSimulation (egs++/egs_application.cpp:839-917, the loop over
// simulateSingleShower and EGS_AdvancedApplication::shower,
// egs++/egs_advanced_application.cpp:871-893) is replaced by one egsgpu_run
// over the same geometry, media and source; everything else -- input parsing,
// geometry and source construction, HATCH, output -- stays the reference's.
//
// It compiles against the reference's egs++ headers and links against the
// reference's egs++ library, its Fortran core and libegsgpu.so, in an egs++
// application directory (with this directory's array_sizes.h).  Here it is
// only compiled (oracle/Makefile, target `ref`) to keep it in step with both
// interfaces.
#include <cstdio>
#include <string>
#include <vector>

#include "egs_advanced_application.h"
#include "egs_base_source.h"
#include "egs_functions.h"
#include "egs_input.h"
#include "egs_interface2.h"
#include "geometry/egs_nd_geometry/egs_nd_geometry.h"

#include "egsgpu.h"

class EGS_GPUDoseApplication : public EGS_AdvancedApplication {
public:
    EGS_GPUDoseApplication(int argc, char **argv) : EGS_AdvancedApplication(argc, argv) {}

    ~EGS_GPUDoseApplication() {
        if (h) egsgpu_destroy(h);
    }

    // The media, geometry and cut-offs after the reference's own initialisation
    // (initSimulation: geometry, source, egsHatch) go to the GPU engine.
    int initSimulation() override {
        int err = EGS_AdvancedApplication::initSimulation();
        if (err) return err;
        EGS_XYZGeometry *g = dynamic_cast<EGS_XYZGeometry *>(geometry);
        if (!g) {
            egsWarning("EGS_GPUDoseApplication: the simulation geometry must be an EGS_XYZGeometry\n");
            return 10;
        }
        egsgpu_config cfg;
        egsgpu_default_config(&cfg);
        cfg.precision = 32;
        cfg.ecut = the_bounds->ecut;   // global ECUT / PCUT of the transport parameter block
        cfg.pcut = the_bounds->pcut;
        if (egsgpu_create(&cfg, &h)) {
            egsWarning("EGS_GPUDoseApplication: no CUDA device\n");
            return 11;
        }
        std::vector<const char *> names;
        for (int m = 0; m < EGS_BaseGeometry::nMedia(); ++m) names.push_back(EGS_BaseGeometry::getMediumName(m));
        std::string data = egsJoinPath(hen_house, "data");
        std::string pegs = egsJoinPath(egsJoinPath(hen_house, "pegs4"), "data");
        pegs = egsJoinPath(pegs, pegs_file + ".pegs4dat");
        if (check(egsgpu_load_media(h, data.c_str(), pegs.c_str(), names.data(), (int)names.size()))) return 12;
        const int nx = g->getNx(), ny = g->getNy(), nz = g->getNz();
        const long long nreg = (long long)nx * ny * nz;
        std::vector<double> xb(g->getXPositions(), g->getXPositions() + nx + 1);
        std::vector<double> yb(g->getYPositions(), g->getYPositions() + ny + 1);
        std::vector<double> zb(g->getZPositions(), g->getZPositions() + nz + 1);
        std::vector<int32_t> med(nreg);
        std::vector<double> rhor(nreg);
        for (long long i = 0; i < nreg; ++i) {
            med[i] = g->medium((int)i);
            rhor[i] = g->getRelativeRho((int)i);
        }
        if (check(egsgpu_set_xyz_geometry(h, nx, ny, nz, xb.data(), yb.data(), zb.data(), med.data(), rhor.data())))
            return 13;
        dose.assign(nreg, 0.0);
        sigma.assign(nreg, 0.0);
        return 0;
    }

    // egsgpu_set_source is given the parallel-beam description this
    // application reads from its own input block (egs_gpu_app.cpp translates
    // the egs++ source blocks the same way); then the whole run is one call.
    int runSimulation() override {
        if (!h || !have_source) {
            egsWarning("EGS_GPUDoseApplication: no GPU source\n");
            return 20;
        }
        if (check(egsgpu_set_source(h, &gpu_source))) return 21;
        if (check(egsgpu_run(h, 0, ncase, nbatch, (uint32_t)i_parallel + 1u, nullptr))) return 22;
        if (check(egsgpu_get_dose(h, dose.data(), sigma.data()))) return 23;
        return 0;
    }

    // Set by the application's input reading: the source in the C ABI's terms.
    egsgpu_source gpu_source = {};
    bool have_source = false;
    long long ncase = 0;
    int nbatch = 10;
    std::vector<double> dose, sigma;

private:
    egsgpu_handle *h = nullptr;
    int check(int st) {
        if (st) egsWarning("egsgpu: %s\n", egsgpu_last_error(h));
        return st;
    }
};

APP_MAIN(EGS_GPUDoseApplication)
