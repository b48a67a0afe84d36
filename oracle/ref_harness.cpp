// Reference harness: a thin extern "C" shell around the reference's OWN
// templates (Integrator::integrate, Lensing::dbetadtheta_infinitesimal,
// Hmaps::FillMap, SimpleHyperOctree::{locate,cic,tsc}, SimpleHyperOctreeIndex
// ::{compute,cipher}, Input::{acquire,correct,load}).  It is TEST
// INFRASTRUCTURE: built by oracle/build_ref.sh into oracle/_ref/ from the
// sources under the reference tree, loaded by tests/golden/make_golden.py and
// by CPU tests through ctypes, and never linked into the product.
//
// The hmaps driver needs HEALPix only for pix2vec_ring (hmaps.h:599); the
// harness supplies its own RING-scheme implementation (Gorski et al. 2005,
// ApJ 622, 759, eqs. 4-10), the same formulas the CUDA map kernel uses, so
// pixel->direction is consistent on both sides but not pinned to libhealpix.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>
#include <array>
#include <map>
#include <sstream>
#include <atomic>
#include <thread>
#include <mpi.h>

// pix2vec_ring, RING scheme, written from the published formulas.
static inline void harness_pix2vec_ring(long nside, long ipix, double* vec)
{
    const double ns = (double)nside;
    const long ncap = 2 * nside * (nside - 1);
    const long npix = 12 * nside * nside;
    double z, phi;
    if (ipix < ncap) {                       // north polar cap
        const long iring = (long)((1 + (long)std::sqrt((double)(1 + 2 * ipix))) / 2);
        long ir = iring;
        // guard the integer square root against rounding
        while (2 * ir * (ir - 1) > ipix) --ir;
        while (2 * (ir + 1) * ir <= ipix) ++ir;
        const long iphi = ipix - 2 * ir * (ir - 1) + 1;
        z = 1.0 - (double)(ir * ir) / (3.0 * ns * ns);
        phi = ((double)iphi - 0.5) * (M_PI / (2.0 * (double)ir));
    } else if (ipix < npix - ncap) {         // equatorial belt
        const long ip = ipix - ncap;
        const long iring = ip / (4 * nside) + nside;
        const long iphi = ip % (4 * nside) + 1;
        const double fodd = ((iring + nside) & 1) ? 1.0 : 0.5;
        z = (2.0 * ns - (double)iring) * 2.0 / (3.0 * ns);
        phi = ((double)iphi - fodd) * (M_PI / (2.0 * ns));
    } else {                                 // south polar cap
        const long ip = npix - ipix;
        long ir = (long)((1 + (long)std::sqrt((double)(2 * ip - 1))) / 2);
        while (2 * ir * (ir - 1) >= ip) --ir;
        while (2 * (ir + 1) * ir < ip) ++ir;
        const long iphi = 4 * ir + 1 - (ip - 2 * ir * (ir - 1));
        z = -1.0 + (double)(ir * ir) / (3.0 * ns * ns);
        phi = ((double)iphi - 0.5) * (M_PI / (2.0 * (double)ir));
    }
    const double st = std::sqrt((1.0 - z) * (1.0 + z));
    vec[0] = st * std::cos(phi);
    vec[1] = st * std::sin(phi);
    vec[2] = z;
}
static inline void pix2vec_ring(long nside, long ipix, double* vec) { harness_pix2vec_ring(nside, ipix, vec); }
static inline long nside2npix(long nside) { return 12 * nside * nside; }

using uint = unsigned int;
using real = double;
using point = std::array<real, 3>;

#include "magrathea/simplehyperoctree.h"
#include "magrathea/simplehyperoctreeindex.h"
#include "magrathea/evolution.h"
#include "magrathea/filelist.h"
#include "cone.h"
#include "utility.h"
#include "input.h"
#include "integrator.h"
#include "lensing.h"
#ifndef VELOCITYFIELD
#include "gravity.h"
#endif
#include "miscellaneous.h"
#include "hmaps.h"
// catalogues.h defines a parameters_t struct and a global `parameters` of
// its own, as hmaps.h does; its dependencies are all in already, so it is
// read with both names renamed.
#define parameters_t catalogues_parameters_t
#define parameters catalogues_parameters
#include "catalogues.h"
#undef parameters
#undef parameters_t

using namespace magrathea;
using Index = SimpleHyperOctreeIndex<__uint128_t, 3>;
using Oct = SimpleHyperOctree<double, Index, Gravity<float, 3>, 3, std::ratio<0>, std::ratio<EXTENT>>;
using Traj = Evolution<Photon<double, 3>>;
using Cosmo = std::array<std::vector<double>, 4>;

static Oct g_octree;
static Cosmo g_cosmo;
static double g_length = 0.0;
// observer velocity of ref_integrate / ref_trajectory / ref_fillmap (read by
// the velocity-field build only, integrator.h:537-538, 707-708)
static std::array<double, 3> g_vobs{0, 0, 0};

struct CosmoParams { std::string celldir, paramfile, evolfile; double mpc = 3.08568E22; };

static void split(__uint128_t k, uint64_t* out)
{
    out[0] = (uint64_t)(k >> 64);
    out[1] = (uint64_t)k;
}

static void data7(const Gravity<float, 3>& d, float* out)
{
    out[0] = d.rho(); out[1] = d.phi(); out[2] = d.dphidx(); out[3] = d.dphidy();
    out[4] = d.dphidz(); out[5] = d.a(); out[6] = d.dphidt();
}

// Photon record, in this order: a t x y z dtdl dxdl dydl dzdl level ah rho phi
// dphidx dphidy dphidz dphidt dphidl laplacian redshift dsdl2 error isw iswold
// chi lambda s index   (28 doubles)
static void photon28(const Photon<double, 3>& p, double* o)
{
    o[0] = p.a(); o[1] = p.t(); o[2] = p.x(); o[3] = p.y(); o[4] = p.z();
    o[5] = p.dtdl(); o[6] = p.dxdl(); o[7] = p.dydl(); o[8] = p.dzdl();
    o[9] = p.level(); o[10] = p.ah(); o[11] = p.rho(); o[12] = p.phi();
    o[13] = p.dphidx(); o[14] = p.dphidy(); o[15] = p.dphidz(); o[16] = p.dphidt();
    o[17] = p.dphidl(); o[18] = p.laplacian(); o[19] = p.redshift(); o[20] = p.dsdl2();
    o[21] = p.error(); o[22] = p.isw(); o[23] = p.iswold(); o[24] = p.chi();
    o[25] = p.lambda(); o[26] = p.s(); o[27] = (double)p.index();
}

template <class F> static void run_threads(int64_t n, int nthreads, F f)
{
    if (nthreads <= 1) { for (int64_t i = 0; i < n; ++i) f(i); return; }
    std::atomic<int64_t> next(0);
    std::vector<std::thread> pool;
    for (int t = 0; t < nthreads; ++t)
        pool.emplace_back([&]() { for (int64_t i; (i = next.fetch_add(1)) < n;) f(i); });
    for (auto& th : pool) th.join();
}

extern "C" {

int ref_extent() { return EXTENT; }
int ref_order() { return ORDER; }

int ref_velocityfield()
{
#ifdef VELOCITYFIELD
    return 1;
#else
    return 0;
#endif
}

void ref_set_vobs(double vx, double vy, double vz) { g_vobs = {vx, vy, vz}; }

int64_t ref_load(const char* path)
{
    g_octree.fullclear();
#ifdef VELOCITYFIELD
    // the reference's cone loader of the velocity-field build: Input::load of
    // the 48-byte records into the wider cells, then the field remap
    // (miscellaneous.h:422-449)
    std::vector<std::string> files{std::string(path)};
    Miscellaneous::loadOctree(0u, g_octree, files);
    if (g_octree.size() == 0) return -1;
#else
    if (!Input::load(g_octree, std::string(path))) return -1;
#endif
    return (int64_t)g_octree.size();
}

int64_t ref_size() { return (int64_t)g_octree.size(); }

void ref_keys(uint64_t* out)
{
    for (size_t i = 0; i < g_octree.size(); ++i) split(std::get<0>(g_octree[i])(), out + 2 * i);
}

void ref_compute(unsigned lvl, double x, double y, double z, uint64_t* out)
{
    split(Index::compute<double, std::ratio<0>, std::ratio<EXTENT>>(lvl, x, y, z)(), out);
}

void ref_cipher(double x, double y, double z, uint64_t* out)
{
    split(Index::cipher<double, std::ratio<0>, std::ratio<EXTENT>>(x, y, z)(), out);
}

unsigned ref_key_level(uint64_t hi, uint64_t lo)
{
    return Index((((__uint128_t)hi) << 64) | lo).level();
}

double ref_key_center(uint64_t hi, uint64_t lo, unsigned dim)
{
    return Index((((__uint128_t)hi) << 64) | lo).center<double, std::ratio<0>, std::ratio<EXTENT>>(dim);
}

int ref_key_containing(uint64_t ahi, uint64_t alo, uint64_t bhi, uint64_t blo)
{
    return Index((((__uint128_t)ahi) << 64) | alo).containing(Index((((__uint128_t)bhi) << 64) | blo));
}

// Index of the located element, or -1 when locate() returns end().
int64_t ref_locate(double x, double y, double z)
{
    auto it = g_octree.locate(x, y, z);
    return (it == g_octree.end()) ? -1 : (int64_t)(it - g_octree.begin());
}

void ref_batch_locate(int64_t n, const double* xyz, int64_t* out, int nthreads)
{
    run_threads(n, nthreads, [&](int64_t i) { out[i] = ref_locate(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]); });
}

void ref_batch_ngp(int64_t n, const double* xyz, float* out, int nthreads)
{
    run_threads(n, nthreads, [&](int64_t i) { data7(g_octree.ngp(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]), out + 7 * i); });
}

void ref_batch_cic(int64_t n, const double* xyz, float* out, int nthreads)
{
    run_threads(n, nthreads, [&](int64_t i) { data7(g_octree.cic(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]), out + 7 * i); });
}

void ref_batch_tsc(int64_t n, const double* xyz, float* out, int nthreads)
{
    run_threads(n, nthreads, [&](int64_t i) {
        std::vector<std::pair<Index, Gravity<float, 3>>> cache(27);
        data7(g_octree.tsc(cache, xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]), out + 7 * i);
    });
}

// Sequential cached TSC over a list of points sharing one 27-cell cache, as the
// integrator does along a ray (simplehyperoctree.h:1552-1644).
void ref_seq_tsc(int64_t n, const double* xyz, float* out)
{
    std::vector<std::pair<Index, Gravity<float, 3>>> cache(27);
    for (int64_t i = 0; i < n; ++i) data7(g_octree.tsc(cache, xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]), out + 7 * i);
}

// Cosmology table as hmaps/catalogues/rays build it: Input::acquire, an FLRW
// ray through a homogeneous level-5 octree (integrate<-1>), Input::correct
// (hmaps.cpp:157-173).  Returns the table size, or -1.
int64_t ref_cosmology(const char* celldir, const char* paramfile, const char* evolfile, double* hol)
{
    CosmoParams p;
    p.celldir = celldir; p.paramfile = paramfile; p.evolfile = evolfile;
    double h = 0, om = 0, lbox = 0;
    Cosmo cosmology = Input::acquire(p, h, om, lbox);
    if (std::get<0>(cosmology).empty()) return -1;
    const double length = lbox * p.mpc / h;
    Oct octree;
    Traj reference;
    const std::array<double, 3> v0{0, 0, 0};
    Input::homogenize(octree.assign(5, 0));
    reference.append(Integrator::launch(0., 0., 0., 0. + EXTENT / 2., 0., 0.));
    Integrator::integrate<-1>(reference, cosmology, octree, v0, length,
        EXTENT * std::pow(2., (uint)(std::log2(std::get<0>(cosmology).size() / std::pow(2., 5) + 1) + 1) + 1));
    g_cosmo = Input::correct(cosmology, reference);
    g_length = length;
    hol[0] = h; hol[1] = om; hol[2] = lbox; hol[3] = length;
    return (int64_t)std::get<0>(g_cosmo).size();
}

void ref_cosmology_get(double* t, double* a, double* dadt, double* d2adt2)
{
    const size_t n = std::get<0>(g_cosmo).size();
    for (size_t i = 0; i < n; ++i) {
        t[i] = g_cosmo[0][i]; a[i] = g_cosmo[1][i]; dadt[i] = g_cosmo[2][i]; d2adt2[i] = g_cosmo[3][i];
    }
}

void ref_cosmology_set(int64_t n, const double* t, const double* a, const double* dadt, const double* d2adt2, double length)
{
    for (int k = 0; k < 4; ++k) g_cosmo[k].assign((size_t)n, 0.0);
    for (int64_t i = 0; i < n; ++i) {
        g_cosmo[0][i] = t[i]; g_cosmo[1][i] = a[i]; g_cosmo[2][i] = dadt[i]; g_cosmo[3][i] = d2adt2[i];
    }
    g_length = length;
}

double ref_interpolate(double x0, int col)
{
    return Utility::interpolate(x0, g_cosmo[0], g_cosmo[col]);
}

// One ray per launch record (x0 y0 z0 x1 y1 z1, the 6-argument
// Integrator::launch), integrated with the stop criterion, then the
// infinitesimal Jacobian at each distance in dists (lensing.h:399-472).
// final28: photon record of trajectory.back(); jac: per distance a11 a12 a21 a22.
void ref_integrate(int64_t n, const double* launch, const char* stop, double stop_ref, unsigned nsteps,
                   int ndist, const double* dists, int64_t* steps, double* final28, double* jac, int nthreads)
{
    const std::string stop_s(stop);
    const std::array<double, 3> v0 = g_vobs;
    run_threads(n, nthreads, [&](int64_t i) {
        const double* L = launch + 6 * i;
        Traj traj;
        traj.append(Integrator::launch(L[0], L[1], L[2], L[3], L[4], L[5]));
        Integrator::integrate(traj, stop_s, stop_ref, g_cosmo, g_octree, v0, g_length, nsteps);
        steps[i] = (int64_t)traj.size();
        if (!traj.empty()) photon28(traj.back(), final28 + 28 * i);
        if (ndist > 0 && traj.size() > 0) {
            std::vector<double> d(dists, dists + ndist);
            auto J = Lensing::dbetadtheta_infinitesimal(d, traj, g_octree, g_length);
            for (int j = 0; j < ndist; ++j) {
                double* o = jac + 4 * (i * ndist + j);
                o[0] = J[j][0][0]; o[1] = J[j][0][1]; o[2] = J[j][1][0]; o[3] = J[j][1][1];
            }
        }
    });
}

// Whole trajectory of one ray (28 doubles per step); returns its size.
int64_t ref_trajectory(const double* L, const char* stop, double stop_ref, unsigned nsteps, double* out, int64_t cap)
{
    const std::array<double, 3> v0 = g_vobs;
    Traj traj;
    traj.append(Integrator::launch(L[0], L[1], L[2], L[3], L[4], L[5]));
    Integrator::integrate(traj, std::string(stop), stop_ref, g_cosmo, g_octree, v0, g_length, nsteps);
    const int64_t m = (int64_t)traj.size();
    for (int64_t k = 0; k < m && k < cap; ++k) photon28(traj[k], out + 28 * k);
    return m;
}

// Homogeneous (FLRW) quantities at each redshift, as hmaps.cpp:302-333 derives
// them from the reference ray: out[5*i..] = t, chi, lambda, a, z.
int ref_homogeneous(int nz, const double* zs, double* out)
{
    Oct octree;
    Traj reference;
    const std::array<double, 3> v0{0, 0, 0};
    Input::homogenize(octree.assign(5, 0));
    reference.append(Integrator::launch(0., 0., 0., 0. + EXTENT / 2., 0., 0.));
    Integrator::integrate<-1>(reference, g_cosmo, octree, v0, g_length,
        EXTENT * std::pow(2., (uint)(std::log2(std::get<0>(g_cosmo).size() / std::pow(2., 5) + 1) + 1) + 1));
    Photon<double, 3> photon;
    for (int i = 0; i < nz; ++i) {
        photon.redshift() = zs[i];
        const unsigned long marked = std::distance(std::begin(reference), std::upper_bound(std::begin(reference), std::end(reference), photon,
            [](const Photon<double, 3>& a, const Photon<double, 3>& b) { return a.redshift() < b.redshift(); }));
        const unsigned long firstid = marked - (marked > 0);
        if (firstid + 1 >= reference.size()) return -1;
        const double f = (reference[firstid + 1].redshift() - zs[i]) / (reference[firstid + 1].redshift() - reference[firstid].redshift());
        out[5 * i + 0] = reference[firstid].t() * f + reference[firstid + 1].t() * (1 - f);
        out[5 * i + 1] = reference[firstid].chi() * f + reference[firstid + 1].chi() * (1 - f);
        out[5 * i + 2] = reference[firstid].lambda() * f + reference[firstid + 1].lambda() * (1 - f);
        out[5 * i + 3] = 1. / (1. + zs[i]);
        out[5 * i + 4] = zs[i];
    }
    return 0;
}

// Hmaps::FillMap (hmaps.h:579-836) itself, with map_components = "lensing"
// (infinitesimal Jacobian) plus the per-pixel extras requested in comps
// (a comma list among dr dl dt da dz ds isw dens dens_max steps phi
// deflection), one ray per pixel of `pixels`.  maps: nmaps*nz rows of npix
// floats, row-major, the layout of the reference's map vector.
int ref_fillmap_jac(long nside, int nz, const double* zvals, const char* stop_ray, const char* comps, unsigned nsteps,
                    int64_t npixels, const long* pixels, float* maps, int* nmaps_out, const char* jacobiantype,
                    const char* plane, const char* stop_bundle, double openingmin)
{
    parameters.nside = nside;
    parameters.nb_z_maps = nz;
    parameters.nsteps = nsteps;
    parameters.stop_ray = stop_ray;
    parameters.jacobiantype = jacobiantype;
    parameters.plane = plane;
    parameters.stop_bundle = stop_bundle;
    parameters.openingmin = openingmin;
    const bool bundle = parameters.jacobiantype == "bundle";
    parameters.map_components = comps;
    std::vector<std::string> map_components;
    {
        std::string cur;
        for (const char c : parameters.map_components) {
            if (c == ',' || c == ' ') { if (!cur.empty()) map_components.push_back(cur); cur.clear(); }
            else cur.push_back(c);
        }
        if (!cur.empty()) map_components.push_back(cur);
    }
    std::vector<uint> index_components(map_components.size());
    static const std::map<std::string, uint> ids = {
        {"lensing", 0}, {"lensing_born", 1}, {"dr", 2}, {"dl", 3}, {"dt", 4}, {"da", 5}, {"dz", 6}, {"ds", 7},
        {"isw", 8}, {"dens", 9}, {"dens_max", 10}, {"steps", 11}, {"phi", 12}, {"deflection", 13}};
    uint nmaps = 0;
    for (size_t i = 0; i < map_components.size(); ++i) {
        auto it = ids.find(map_components[i]);
        if (it == ids.end()) return -1;
        index_components[i] = it->second;
        // rows per component as hmaps.cpp:196-250 counts them
        nmaps += (it->second == 0) ? (bundle ? 5 : 4) : (it->second == 1) ? 4 : (it->second == 13 ? 2 : 1);
    }
    *nmaps_out = (int)nmaps;
    std::vector<double> hom(5 * (size_t)nz);
    std::vector<double> zs(zvals, zvals + nz);
    if (ref_homogeneous(nz, zvals, hom.data()) != 0) return -2;
    std::vector<double> thomo(nz), rhomo(nz), lambdahomo(nz), ahomo(nz), redshifthomo(nz);
    for (int i = 0; i < nz; ++i) {
        thomo[i] = hom[5 * i]; rhomo[i] = hom[5 * i + 1]; lambdahomo[i] = hom[5 * i + 2];
        ahomo[i] = hom[5 * i + 3]; redshifthomo[i] = hom[5 * i + 4];
    }
    std::vector<double> interpRefvec;
    const std::string s(stop_ray);
    if (s == "t") interpRefvec = thomo;
    else if (s == "r" || s == "s") interpRefvec = rhomo;
    else if (s == "lambda") interpRefvec = lambdahomo;
    else if (s == "a") interpRefvec = ahomo;
    else if (s == "redshift") interpRefvec = zs;
    else return -3;
    // pixel ids are used as map offsets: remap them to 0..npixels-1 rows
    std::vector<long> pix(pixels, pixels + npixels);
    long maxpix = 0;
    for (long p : pix) maxpix = std::max(maxpix, p);
    std::vector<std::vector<float>> map((size_t)nmaps * nz, std::vector<float>((size_t)maxpix + 1, 0.f));
    const std::array<double, 3> v0 = g_vobs;   // the map driver's vobs (hmaps.cpp:364, 450)
    const point observer{{0., 0., 0.}};
    Hmaps::FillMap(parameters, map_components, index_components, (unsigned)npixels, 0u, g_octree, v0, map, nmaps, pix,
                   g_cosmo, observer, g_length, interpRefvec, rhomo, thomo, lambdahomo, redshifthomo, ahomo);
    for (size_t r = 0; r < map.size(); ++r)
        for (int64_t k = 0; k < npixels; ++k) maps[r * npixels + k] = map[r][pix[k]];
    return 0;
}

int ref_fillmap(long nside, int nz, const double* zvals, const char* stop_ray, const char* comps, unsigned nsteps,
                int64_t npixels, const long* pixels, float* maps, int* nmaps_out)
{
    return ref_fillmap_jac(nside, nz, zvals, stop_ray, comps, nsteps, npixels, pixels, maps, nmaps_out, "infinitesimal",
                           "normal", "redshift", 0.0);
}

void ref_pix2vec_ring(long nside, int64_t n, const long* pix, double* vec)
{
    for (int64_t i = 0; i < n; ++i) harness_pix2vec_ring(nside, pix[i], vec + 3 * i);
}

// Catalogues::relCat's per-source work (catalogues.h:811-856): the source
// position and velocity (rotated by rotm1 unless it is null, the full-sky
// case), the comoving first guess, Catalogues::iterateNewtonMethod with the
// infinitesimal Jacobian, and the 16-double catalog row.
// src: n x 6 (x y z vx vy vz); rotm1: 3x3 row-major or null; vobs: 3;
// out: n x 16.
void ref_catalogue_jac(int64_t n, const double* src, const double* rotm1, const double* vobs, double cat_accuracy,
                       unsigned nsteps, double h, double mpc, double* out, int nthreads, const char* jacobiantype,
                       const char* plane, const char* stop_bundle, double openingmin)
{
    catalogues_parameters_t P;
    P.isfullsky = rotm1 ? 0 : 1;
    P.mpc = mpc;
    P.cat_accuracy = cat_accuracy;
    P.jacobiantype = jacobiantype;
    P.plane = plane;
    P.stop_bundle = stop_bundle;
    P.nsteps = nsteps;
    P.use_previous_catalogues = 0;
    P.openingmin = openingmin;
    const point vo{{vobs[0], vobs[1], vobs[2]}};
    const point observer{{0., 0., 0.}};
    std::array<std::array<double, 3>, 3> rot{};
    if (rotm1)
        for (int j = 0; j < 3; ++j)
            for (int k = 0; k < 3; ++k) rot[j][k] = rotm1[3 * j + k];
    run_threads(n, nthreads, [&](int64_t i) {
        const double* s = src + 6 * i;
        point trueTarget, velocityTarget;
        for (unsigned j = 0; j < 3; j++) {
            if (P.isfullsky == 1) {
                trueTarget[j] = s[j];
                velocityTarget[j] = s[j + 3];
            } else {
                trueTarget[j] = s[0] * rot[j][0] + s[1] * rot[j][1] + s[2] * rot[j][2];
                velocityTarget[j] = s[3] * rot[j][0] + s[4] * rot[j][1] + s[5] * rot[j][2];
            }
        }
        std::array<std::array<double, 2>, 2> jacobian;
        double interpRef = 0;
        std::vector<double> redshifts(6);
        const double distTarget = std::sqrt(trueTarget[0] * trueTarget[0] + trueTarget[1] * trueTarget[1] +
                                            trueTarget[2] * trueTarget[2]);
        const double theta = std::acos(trueTarget[2] / distTarget);
        const double phi = std::atan2(trueTarget[1], trueTarget[0]);
        // (newtonMethod2d leaves result[1][1] unset when a bundle Jacobian
        // fails, catalogues.h:525-529, 670-675: that column is undefined there)
        auto result = Catalogues::iterateNewtonMethod(vo, observer, phi, theta, trueTarget, velocityTarget, jacobian, P,
                                                      g_cosmo, g_octree, g_length, h, redshifts, interpRef);
        double* o = out + 16 * i;
        o[0] = phi; o[1] = theta;
        o[2] = result[0][0]; o[3] = result[0][1]; o[4] = result[1][0]; o[5] = result[1][1];
        for (int k = 0; k < 6; ++k) o[6 + k] = redshifts[k];
        o[12] = jacobian[0][0]; o[13] = jacobian[0][1]; o[14] = jacobian[1][0]; o[15] = jacobian[1][1];
    });
}

void ref_catalogue(int64_t n, const double* src, const double* rotm1, const double* vobs, double cat_accuracy,
                   unsigned nsteps, double h, double mpc, double* out, int nthreads)
{
    ref_catalogue_jac(n, src, rotm1, vobs, cat_accuracy, nsteps, h, mpc, out, nthreads, "infinitesimal", "normal", "r", 0.0);
}

// Integrator::propagate (integrator.h:861-1015): the launched photon L (start
// x y z, end x y z) and `count` photons on a circle of half-angle `angle`
// around it (rotated by `rotation`), each integrated with the no-stop
// Integrator::integrate, the bundle checks, and the central ray's angular
// diameter distance.  out: up to cap points x 29 in the trajectory file's
// column order (photon_file29); text (up to text_cap bytes, NUL-terminated)
// receives Output::save of the central trajectory at max_digits10, as the rays
// driver writes it (output.h:200-211).  Returns the central trajectory's size,
// 0 when the bundle is rejected.
static void photon_file29(const Photon<double, 3>& p, double* o)
{
    o[0] = (double)p.index(); o[1] = p.a(); o[2] = p.t(); o[3] = p.x(); o[4] = p.y(); o[5] = p.z();
    o[6] = p.dtdl(); o[7] = p.dxdl(); o[8] = p.dydl(); o[9] = p.dzdl();
    o[10] = p.level(); o[11] = p.ah(); o[12] = p.rho(); o[13] = p.phi();
    o[14] = p.dphidx(); o[15] = p.dphidy(); o[16] = p.dphidz(); o[17] = p.dphidl(); o[18] = p.laplacian();
    o[19] = p.redshift(); o[20] = p.dsdl2(); o[21] = p.error(); o[22] = p.distance();
    o[23] = p.isw(); o[24] = p.iswold(); o[25] = p.chi(); o[26] = p.lambda(); o[27] = p.dphidt(); o[28] = p.s();
}

int64_t ref_propagate_bundle(const double* L, unsigned count, double angle, double rotation, const char* interp,
                             double amin, unsigned nsteps, double* out, int64_t cap, char* text, int64_t text_cap)
{
    const std::array<double, 3> v0{0, 0, 0};
    const Photon<double, 3> ph = Integrator::launch(L[0], L[1], L[2], L[3], L[4], L[5]);
    Traj t = Integrator::propagate(ph, count, angle, rotation, std::string(interp), g_cosmo, g_octree, v0, g_length,
                                   nsteps, amin);
    const int64_t m = (int64_t)t.size();
    for (int64_t k = 0; k < m && k < cap; ++k) photon_file29(t[k], out + 29 * k);
    if (text && text_cap > 0) {
        std::ostringstream os;
        Output::save(os, t, std::numeric_limits<double>::max_digits10);
        const std::string str = os.str();
        const size_t n = std::min<size_t>(str.size(), (size_t)text_cap - 1);
        std::memcpy(text, str.data(), n);
        text[n] = 0;
    }
    return m;
}

// The FLRW reference bundle of the rays driver (rays.cpp:244-249): the same
// Integrator::propagate at Order = -1 on a uniform octree of `level`
// (homotree.assign(level, 0)).  Output as ref_propagate_bundle.
int64_t ref_propagate_bundle_flrw(const double* L, unsigned count, double angle, const char* interp, unsigned nsteps,
                                  unsigned level, double* out, int64_t cap)
{
    const std::array<double, 3> v0{0, 0, 0};
    Oct homotree;
    homotree.assign(level, 0);
    const Photon<double, 3> ph = Integrator::launch(L[0], L[1], L[2], L[3], L[4], L[5]);
    Traj t = Integrator::propagate<-1>(ph, count, angle, 0.0, std::string(interp), g_cosmo, homotree, v0, g_length,
                                       nsteps, 0.0);
    const int64_t m = (int64_t)t.size();
    for (int64_t k = 0; k < m && k < cap; ++k) photon_file29(t[k], out + 29 * k);
    return m;
}

// create_octree for one cone from one ASCII cell file (Create_octree::
// PreparationASCII, create_octree.h:544-580): Input::importascii with the
// reference's cone / sphere collision filter (input.h:996-1067, 216-226),
// then Miscellaneous::correctOctree (miscellaneous.h:467-479: sistemize,
// dphidt = 0, Input::correct, dphidt *= da/dt(a)) on the loaded cosmology.
// cone7: vertex xyz, base xyz, angle; sphere4: centre xyz, radius; rotm1:
// 3x3 row-major or NULL (full sky).  out: up to cap 48-byte records (what
// Input::save writes).  Returns the cell count; *amin_out receives amin.
struct HarnessBuildParams {
    unsigned isfullsky, coarseonly, ncoarse, correction, coarsecorrection, acorrection;
    double mpc;
};

int64_t ref_build_cone(const char* cellfile, const double* cone7, const double* sphere4, const double* rotm1,
                       unsigned coarseonly, unsigned ncoarse, unsigned correction, unsigned coarsecorrection,
                       unsigned acorrection, double mpc, double h, double omegam, double lboxmpch, void* out, int64_t cap,
                       double* amin_out)
{
    HarnessBuildParams prm{rotm1 ? 0u : 1u, coarseonly, ncoarse, correction, coarsecorrection, acorrection, mpc};
    std::array<std::array<double, 3>, 3> rot = {{{0, 0, 0}}};
    if (rotm1)
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) rot[r][c] = rotm1[3 * r + c];
    const point vertex{cone7[0], cone7[1], cone7[2]}, base{cone7[3], cone7[4], cone7[5]};
    const Cone<point> cone(vertex, base, cone7[6]);
    const HyperSphere<3, point> sphere(point{sphere4[0], sphere4[1], sphere4[2]}, sphere4[3]);
    Oct octree;
    using Element = std::remove_cv<std::remove_reference<decltype(octree[0])>::type>::type;
    Input::importascii<std::ratio<0>, std::ratio<EXTENT>>(prm, rot, octree, std::string(cellfile),
                                                          [&](const Element& e) { return Input::collide(octree, std::get<0>(e), sphere, cone); });
    double amin = 0.0;
    Miscellaneous::correctOctree(octree, g_cosmo, prm, h, omegam, lboxmpch, amin);
    const int64_t m = (int64_t)octree.size();
    for (int64_t k = 0; k < m && k < cap; ++k) std::memcpy((char*)out + 48 * k, &octree[k], 48);
    if (amin_out) *amin_out = amin;
    return m;
}


#ifdef VELOCITYFIELD
// The velocity-field map driver's particle stage (hmaps.cpp:395-441).
// flags 1: every cell's rho and velocity zeroed (hmaps.cpp:396); then the
// reference's Hmaps::CreateOctreeVelocityWithCIC (scheme 1) / WithTSC
// (scheme 2) over the particles, fed a few particles per call so that its
// Utility::parallelize runs them all on the calling thread, in order (the
// reference's own threads add to shared cells without atomics); flags 2:
// the mass normalisation and the parent fill of hmaps.cpp:424-441, written
// out here because the reference has them inline in main().
int ref_velocity_deposit(int scheme, int64_t n, const float* pos, const float* vel, int flags)
{
    if (flags & 1) {
        for (size_t i = 0; i < g_octree.size(); ++i) {
            std::get<1>(g_octree[i]).rho() = 0;
            std::get<1>(g_octree[i]).vxyz() = std::array<float, 3>();
        }
    }
    const unsigned hw = std::thread::hardware_concurrency();
    const int64_t chunk = (hw > 1) ? (int64_t)hw - 1 : 1;
    for (int64_t lo = 0; lo < n; lo += chunk) {
        const int64_t m = std::min<int64_t>(chunk, n - lo);
        std::vector<float> p(pos + 3 * lo, pos + 3 * (lo + m)), v(vel + 3 * lo, vel + 3 * (lo + m));
        if (scheme == 1) Hmaps::CreateOctreeVelocityWithCIC(g_octree, p, v);
        else if (scheme == 2) Hmaps::CreateOctreeVelocityWithTSC(g_octree, p, v);
        else return -1;
    }
    if (flags & 2) {
        unsigned lmin = 1000, lmax = 0;
        for (size_t i = 0; i < g_octree.size(); ++i) {
            lmin = std::min(lmin, std::get<0>(g_octree[i]).level());
            lmax = std::max(lmax, std::get<0>(g_octree[i]).level());
        }
        for (size_t i = 0; i < g_octree.size(); ++i) {
            auto& d = std::get<1>(g_octree[i]);
            double mass = d.rho();
            mass = mass + (mass == 0);
            d.vx() /= mass;
            d.vy() /= mass;
            d.vz() /= mass;
        }
        for (unsigned l = lmin + 1; l <= lmax; ++l)
            for (size_t i = 0; i < g_octree.size(); ++i) {
                if (std::get<0>(g_octree[i]).level() != l || std::isnormal(std::get<1>(g_octree[i]).rho())) continue;
                const auto par = g_octree.find(std::get<0>(g_octree[i]).parent());
                if (par == g_octree.end()) continue;
                const auto& pd = std::get<1>(*par);
                std::get<1>(g_octree[i]).vxyz() = {pd.vx(), pd.vy(), pd.vz()};
            }
    }
    return 0;
}

// the cells' velocities (n x 3) and rho (n)
void ref_velocity_get(float* v3, float* rho)
{
    for (size_t i = 0; i < g_octree.size(); ++i) {
        const auto& d = std::get<1>(g_octree[i]);
        v3[3 * i] = d.vx(); v3[3 * i + 1] = d.vy(); v3[3 * i + 2] = d.vz();
        rho[i] = d.rho();
    }
}

// sets the cells' velocities (and rho, if given)
void ref_velocity_set(const float* v3, const float* rho)
{
    for (size_t i = 0; i < g_octree.size(); ++i) {
        auto& d = std::get<1>(g_octree[i]);
        d.vxyz() = {v3[3 * i], v3[3 * i + 1], v3[3 * i + 2]};
        if (rho) d.rho() = rho[i];
    }
}
#endif

}  // extern "C"
