// The reference-side call sites of INTEGRATION.md, compiled as C++17 against
// include/mpf_gb300.h and linked to libmpf_gb300.so: the octree and cosmology
// uploads (hmaps.cpp:346-353), FillMap's map rows (hmaps.h:583-834) and
// relCat's catalogue rows (catalogues.h:803-903) with the reference's own
// container types.  Inputs are raw files written by tests/test_gpu_cpp_boundary.py
// from a golden fixture; outputs are raw files it compares with the
// reference's rows.
//
//   integration_calls <dir>     reads <dir>/*.in, writes <dir>/maps.out and <dir>/catalogue.out
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

int main(int argc, char** argv)
{
    if (argc != 2) {
        std::fprintf(stderr, "usage: %s <dir>\n", argv[0]);
        return 2;
    }
    const std::string dir = argv[1];
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
