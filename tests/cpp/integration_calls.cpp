// The reference-side call sites of INTEGRATION.md, compiled as C++17 against
// include/mpf_gb300.h and linked to libmpf_gb300.so: the octree and cosmology
// uploads (hmaps.cpp:346-353), FillMap's map rows (hmaps.h:583-834) and
// relCat's catalogue rows (catalogues.h:803-903) with the reference's own
// container types.  Inputs are raw files written by tests/test_gpu_cpp_boundary.py
// from a golden fixture; outputs are raw files it compares with the
// reference's rows.
//
//   integration_calls <dir>            reads <dir>/*.in, writes <dir>/maps.out and <dir>/catalogue.out
//   integration_calls <dir> velocity   the velocity-field map driver (hmaps.cpp:360-455): the
//                                      particles of two shell files deposited (TSC), the maps traced
//                                      with the observer velocity; writes velocity.out, rho.out,
//                                      maps.out, and accuracy.out (mpf_propagate_accuracy on the
//                                      pixels' rays)
#include <array>
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "mpf_gb300.h"

template <class T>
static std::vector<T> slurp(const std::string& path)
{
    std::ifstream f(path, std::ios::binary | std::ios::ate);
    if (!f) throw std::runtime_error("cannot read " + path);
    const std::streamsize bytes = f.tellg();
    f.seekg(0);
    std::vector<T> v((size_t)bytes / sizeof(T));
    f.read(reinterpret_cast<char*>(v.data()), (std::streamsize)(v.size() * sizeof(T)));
    return v;
}

template <class T>
static void spill(const std::string& path, const T* p, size_t n)
{
    std::ofstream f(path, std::ios::binary);
    f.write(reinterpret_cast<const char*>(p), (std::streamsize)(n * sizeof(T)));
}

static void check(int rc, const char* what)
{
    if (rc < 0) throw std::runtime_error(std::string(what) + ": " + mpf_last_error());
}

// The velocity-field build's map driver, with the files of the velocity fixture.
static void velocity_driver(const std::string& dir)
{
    struct Record48 {
        unsigned char bytes[48];
    };
    const std::vector<Record48> octree = slurp<Record48>(dir + "/records.in");
    const std::vector<double> table = slurp<double>(dir + "/cosmology.in");
    const size_t nt = table.size() / 4;
    // length, nsteps, nside, v0x, v0y, v0z, first-file particles
    const std::vector<double> s = slurp<double>(dir + "/scalars.in");
    std::vector<double> interpRefvec = slurp<double>(dir + "/surfaces.in");
    std::vector<double> homogeneous = slurp<double>(dir + "/homogeneous.in");
    std::vector<int64_t> pixel = slurp<int64_t>(dir + "/pixels.in");
    const std::vector<float> pos_all = slurp<float>(dir + "/pos.in"), vel_all = slurp<float>(dir + "/vel.in");
    const size_t split = (size_t)s[6];
    // two shell files, as fill_particles_vectors hands them over
    const std::vector<std::vector<float>> pos_part = {std::vector<float>(pos_all.begin(), pos_all.begin() + 3 * split),
                                                      std::vector<float>(pos_all.begin() + 3 * split, pos_all.end())};
    const std::vector<std::vector<float>> vel_part = {std::vector<float>(vel_all.begin(), vel_all.begin() + 3 * split),
                                                      std::vector<float>(vel_all.begin() + 3 * split, vel_all.end())};

    mpf_octree* dtree = nullptr;
    check(mpf_octree_upload(octree.data(), (int64_t)octree.size(), &dtree), "mpf_octree_upload");
    mpf_cosmology* dcosmo = nullptr;
    check(mpf_cosmology_upload(table.data(), table.data() + nt, table.data() + 2 * nt, table.data() + 3 * nt,
                               (int64_t)nt, &dcosmo),
          "mpf_cosmology_upload");
    const int scheme = 2;   // parameters.velocity_field == "tsc"
    bool first = true;
    for (size_t ifile = 0; ifile < pos_part.size(); ++ifile) {
        check(mpf_velocity_deposit(dtree, scheme, (int64_t)(pos_part[ifile].size() / 3), pos_part[ifile].data(),
                                   vel_part[ifile].data(), first ? MPF_VELOCITY_BEGIN : 0),
              "mpf_velocity_deposit");
        first = false;
    }
    check(mpf_velocity_deposit(dtree, scheme, 0, nullptr, nullptr, MPF_VELOCITY_FINISH), "mpf_velocity_deposit");
    std::vector<float> v3(3 * octree.size()), rho(octree.size());
    check(mpf_octree_get_velocity(dtree, v3.data(), rho.data()), "mpf_octree_get_velocity");
    spill(dir + "/velocity.out", v3.data(), v3.size());
    spill(dir + "/rho.out", rho.data(), rho.size());

    mpf_params p = {};
    p.length = s[0];
    p.nsteps = (unsigned)s[1];
    p.order = 2;
    p.stop = MPF_STOP_REDSHIFT;
    p.planes = interpRefvec.data();
    p.nplanes = (int)interpRefvec.size();
    p.jacobian = 1;
    p.exact = 1;
    p.vobs[0] = s[3];
    p.vobs[1] = s[4];
    p.vobs[2] = s[5];
    const std::vector<int> comps = {MPF_MAP_LENSING, MPF_MAP_DZ, MPF_MAP_ISW, MPF_MAP_DENS, MPF_MAP_STEPS};
    const int nmaps = 4 + 4;
    const int64_t npix = (int64_t)pixel.size();
    std::vector<float> rows((size_t)nmaps * interpRefvec.size() * npix);
    check(mpf_hmaps_fill(dtree, dcosmo, &p, (int64_t)s[2], npix, pixel.data(), (int)comps.size(), comps.data(),
                         homogeneous.data(), rows.data()),
          "mpf_hmaps_fill");
    spill(dir + "/maps.out", rows.data(), rows.size());

    // the error the FP32-gather call carries against the float64 run, on the pixels' rays
    std::vector<double> vec(3 * pixel.size()), launch(6 * pixel.size(), 0.0);
    check(mpf_pix2vec_ring((int64_t)s[2], npix, pixel.data(), vec.data()), "mpf_pix2vec_ring");
    for (int64_t i = 0; i < npix; ++i)
        for (int d = 0; d < 3; ++d) launch[6 * i + 3 + d] = vec[3 * i + d];
    mpf_accuracy acc;
    check(mpf_propagate_accuracy(dtree, dcosmo, &p, npix, launch.data(), 64, &acc), "mpf_propagate_accuracy");
    const double a[] = {(double)acc.rays, (double)acc.step_count_differs, acc.deflection_rel_max, acc.redshift_rel_max,
                        acc.lensing_abs_max[0], acc.lensing_scale[0]};
    spill(dir + "/accuracy.out", a, 6);
    mpf_octree_destroy(dtree);
    mpf_cosmology_destroy(dcosmo);
}

int main(int argc, char** argv)
{
    if (argc != 2 && !(argc == 3 && std::string(argv[2]) == "velocity")) {
        std::fprintf(stderr, "usage: %s <dir> [velocity]\n", argv[0]);
        return 2;
    }
    const std::string dir = argv[1];
    if (argc == 3) {
        try {
            velocity_driver(dir);
        } catch (const std::exception& e) {
            std::fprintf(stderr, "integration_calls: %s\n", e.what());
            return 1;
        }
        return 0;
    }
    try {
        // the cone's records as Input::load read them (48-byte key + Gravity<float,3>)
        struct Record48 {
            unsigned char bytes[48];
        };
        const std::vector<Record48> octree = slurp<Record48>(dir + "/records.in");
        // the cosmology table of Input::acquire + Input::correct: t, a, dadt, d2adt2
        const std::vector<double> table = slurp<double>(dir + "/cosmology.in");
        const size_t nt = table.size() / 4;
        std::array<std::vector<double>, 4> cosmology;
        for (int q = 0; q < 4; ++q) cosmology[q].assign(table.begin() + q * nt, table.begin() + (q + 1) * nt);
        // length, h, mpc, nsteps, nside, order, cat_accuracy, vobs x y z
        const std::vector<double> s = slurp<double>(dir + "/scalars.in");
        const double length = s[0], h = s[1], mpc = s[2];
        const unsigned nsteps = (unsigned)s[3];
        const long nside = (long)s[4];
        const int order = (int)s[5];
        const double cat_accuracy = s[6];
        const std::array<double, 3> vobs = {s[7], s[8], s[9]};
        std::vector<double> interpRefvec = slurp<double>(dir + "/surfaces.in");
        std::vector<double> homogeneous = slurp<double>(dir + "/homogeneous.in");   // nz x 5: t chi lambda a z
        std::vector<int64_t> pixel = slurp<int64_t>(dir + "/pixels.in");
        const std::vector<double> src = slurp<double>(dir + "/sources.in");         // n x 8
        std::vector<std::array<double, 8>> targets_position(src.size() / 8);
        for (size_t i = 0; i < targets_position.size(); ++i)
            for (int q = 0; q < 8; ++q) targets_position[i][q] = src[8 * i + q];

        // -- octree and cosmology (once per cone) --
        mpf_octree* dtree = nullptr;
        check(mpf_octree_upload(octree.data(), (int64_t)octree.size(), &dtree), "mpf_octree_upload");
        mpf_cosmology* dcosmo = nullptr;
        check(mpf_cosmology_upload(cosmology[0].data(), cosmology[1].data(), cosmology[2].data(), cosmology[3].data(),
                                   (int64_t)cosmology[0].size(), &dcosmo),
              "mpf_cosmology_upload");

        // -- hmaps: FillMap's rows for the cone's pixels, on the device --
        mpf_params p = {};
        p.length = length;
        p.nsteps = nsteps;
        p.order = order;
        p.stop = MPF_STOP_REDSHIFT;
        p.planes = interpRefvec.data();
        p.nplanes = (int)interpRefvec.size();
        p.jacobian = 1;
        p.exact = 1;
        const std::vector<int> comps = {MPF_MAP_LENSING, MPF_MAP_DR,   MPF_MAP_DZ,  MPF_MAP_ISW,       MPF_MAP_DENS,
                                        MPF_MAP_DENS_MAX, MPF_MAP_STEPS, MPF_MAP_PHI, MPF_MAP_DEFLECTION};
        const int nmaps = 4 + 7 + 2;   // lensing 4 rows, deflection 2, the rest 1
        const int64_t npix = (int64_t)pixel.size();
        std::vector<float> rows((size_t)nmaps * interpRefvec.size() * npix);
        check(mpf_hmaps_fill(dtree, dcosmo, &p, nside, npix, pixel.data(), (int)comps.size(), comps.data(),
                             homogeneous.data(), rows.data()),
              "mpf_hmaps_fill");
        spill(dir + "/maps.out", rows.data(), rows.size());

        // -- catalogues: relCat's rows, the 8-column source rows as they are --
        mpf_catalogue_params cp = {};
        cp.length = length;
        cp.h = h;
        cp.mpc = mpc;
        cp.cat_accuracy = cat_accuracy;
        cp.vobs[0] = vobs[0];
        cp.vobs[1] = vobs[1];
        cp.vobs[2] = vobs[2];
        cp.rotm1 = nullptr;
        cp.nsteps = nsteps;
        cp.order = order;
        cp.exact = 1;
        cp.max_iterations = 10;
        std::vector<std::array<double, 16>> catalog(targets_position.size());
        check(mpf_catalogue_newton(dtree, dcosmo, &cp, (int64_t)targets_position.size(), targets_position[0].data(), 8,
                                   catalog[0].data(), nullptr),
              "mpf_catalogue_newton");
        spill(dir + "/catalogue.out", catalog[0].data(), 16 * catalog.size());

        mpf_octree_destroy(dtree);
        mpf_cosmology_destroy(dcosmo);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "integration_calls: %s\n", e.what());
        return 1;
    }
    return 0;
}
