// C ABI of the photon-propagation path (declarations: include/mpf_gb300.h).
#include <cstdio>
#include <cmath>
#include <algorithm>
#include <map>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/mpf_gb300.h"
#include "mpf_catalogue.h"
#include "mpf_internal.h"
#include "mpf_maps.h"

extern "C" int mpf_internal_octree_build(const void* records, int64_t n, int on_device, cudaStream_t stream,
                                         mpf_octree** out, char* err, int errlen);

namespace mpf {
cudaError_t launch_gather_exact(const DevTree& T, int kind, const double* d_xyz, long long n, void* d_out, cudaStream_t s);
cudaError_t launch_gather_fast(const DevTree& T, int kind, const double* d_xyz, long long n, void* d_out, cudaStream_t s);
}  // namespace mpf

namespace {

thread_local std::string g_err;

int set_err(int code, const std::string& msg)
{
    g_err = msg;
    return code;
}

int cuda_err(cudaError_t e, const char* where)
{
    return set_err(e == cudaErrorMemoryAllocation ? MPF_OUT_OF_MEMORY : MPF_CUDA_ERROR,
                   std::string(where) + ": " + cudaGetErrorString(e));
}

bool has_device()
{
    int n = 0;
    return cudaGetDeviceCount(&n) == cudaSuccess && n > 0;
}

// A non-blocking stream per host thread and device for the host-buffer
// calls: calls from different host threads never share a stream, nor the
// stream's work-queue counter (on the legacy default stream, one thread's
// queue reset could land between another's reset and launch).  Kept for the
// thread's lifetime.
cudaError_t host_stream(cudaStream_t* out)
{
    thread_local std::map<int, cudaStream_t> mine;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    auto it = mine.find(dev);
    if (it == mine.end()) {
        cudaStream_t a = nullptr;
        e = cudaStreamCreateWithFlags(&a, cudaStreamNonBlocking);
        if (e != cudaSuccess) return e;
        it = mine.emplace(dev, a).first;
    }
    *out = it->second;
    return cudaSuccess;
}

// RAII device buffer
struct DBuf {
    void* p = nullptr;
    cudaError_t alloc(size_t bytes)
    {
        if (bytes == 0) return cudaSuccess;
        return cudaMalloc(&p, bytes);
    }
    ~DBuf()
    {
        if (p) cudaFree(p);
    }
};

}  // namespace

// Parameter checks and the device parameter block of every propagation call
// (mpf_propagate, mpf_propagate_device, mpf_propagate_noalloc, the map calls).
bool mpf_internal_fill_params(const mpf_params* p, mpf::PropParams& P)
{
    if (!p || p->nsteps == 0 || p->order < 0 || p->order > 2 || p->stop < 0 || p->stop > 6 || p->nplanes < 0 ||
        p->nplanes > MPF_MAX_PLANES || !(p->length > 0.0))
        return false;
    if (p->nplanes > 0 && !p->planes) return false;
    if (p->nplanes > 0 && p->stop == MPF_STOP_PLANE) return false;
    std::memset(&P, 0, sizeof(P));
    P.length = p->length;
    P.stop_ref = (p->nplanes > 0) ? p->planes[p->nplanes - 1] : p->stop_value;
    for (int k = 0; k < 3; ++k) P.ki[k] = p->plane_normal[k];
    for (int k = 0; k < p->nplanes; ++k) P.planes[k] = p->planes[k];
    P.max_steps = (p->max_steps > 0) ? p->max_steps : 100000000ll;
    P.nsteps = p->nsteps;
    P.order = p->order;
    P.stop_kind = p->stop;
    P.nplanes = p->nplanes;
    P.jacobian = p->jacobian ? 1 : 0;
    for (int k = 0; k < 3; ++k) {
        if (!std::isfinite(p->vobs[k])) return false;
        P.vobs[k] = p->vobs[k];
    }
    return true;
}

namespace {
bool fill_params(const mpf_params* p, mpf::PropParams& P) { return mpf_internal_fill_params(p, P); }
}  // namespace

int mpf_internal_set_error(int code, const char* msg) { return set_err(code, msg ? msg : ""); }

extern "C" {

int mpf_version(void) { return 1; }

const char* mpf_last_error(void) { return g_err.c_str(); }

int mpf_device_count(void)
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
    return n;
}

int mpf_octree_upload(const void* records, int64_t n, mpf_octree** out)
{
    if (!records || n <= 0 || !out) return set_err(MPF_BAD_INPUT, "mpf_octree_upload: null buffer or empty octree");
    if (!has_device()) return set_err(MPF_NO_DEVICE, "mpf_octree_upload: no CUDA device");
    char err[256] = {0};
    const int rc = mpf_internal_octree_build(records, n, 0, 0, out, err, sizeof(err));
    if (rc == 0) return MPF_OK;
    const int code = (rc == -2) ? MPF_OUT_OF_MEMORY : (rc == -3) ? MPF_CUDA_ERROR : (rc == -4) ? MPF_NOT_SORTED : MPF_BAD_INPUT;
    return set_err(code, std::string("mpf_octree_upload: ") + err);
}

int mpf_octree_load(const char* path, mpf_octree** out)
{
    if (!path || !out) return set_err(MPF_BAD_INPUT, "mpf_octree_load: null argument");
    FILE* f = std::fopen(path, "rb");
    if (!f) return set_err(MPF_IO_ERROR, std::string("mpf_octree_load: cannot open ") + path);
    std::fseek(f, 0, SEEK_END);
    const long long size = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    if (size <= 0 || size % 48 != 0) {
        std::fclose(f);
        return set_err(MPF_IO_ERROR, std::string("mpf_octree_load: size is not a multiple of 48 bytes: ") + path);
    }
    std::vector<unsigned char> buf((size_t)size);
    const size_t got = std::fread(buf.data(), 1, (size_t)size, f);
    std::fclose(f);
    if (got != (size_t)size) return set_err(MPF_IO_ERROR, std::string("mpf_octree_load: short read: ") + path);
    return mpf_octree_upload(buf.data(), size / 48, out);
}

int mpf_octree_get_info(const mpf_octree* o, mpf_octree_info* info)
{
    if (!o || !info) return set_err(MPF_BAD_INPUT, "mpf_octree_get_info: null argument");
    info->cells = o->n;
    info->nodes = o->nnodes;
    info->level_min = o->level_min;
    info->level_max = o->level_max;
    info->top_level = o->tree.Lt;
    info->grid[0] = o->tree.gnx;
    info->grid[1] = o->tree.gny;
    info->grid[2] = o->tree.gnz;
    info->device_bytes = o->n * (int64_t)(sizeof(ulonglong2) + 2 * sizeof(float4) + 8 * sizeof(int4)) + o->nnodes * (int64_t)sizeof(int2) +
                         (int64_t)o->tree.gnx * o->tree.gny * o->tree.gnz * (int64_t)sizeof(int);
    return MPF_OK;
}

void mpf_octree_destroy(mpf_octree* o)
{
    if (!o) return;
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(o->device);
    mpf::forget_tuned_shape((const void*)o->tree.keys);
    mpf::catalogue_forget_tuned_shape((const void*)o->tree.keys);
    cudaFree(o->keys);
    cudaFree(o->grad);
    cudaFree(o->scal);
    cudaFree(o->node);
    cudaFree(o->grid);
    cudaFree(o->stencil);
    if (o->vel) cudaFree(o->vel);
    cudaSetDevice(cur);
    delete o;
}

int mpf_cosmology_upload(const double* t, const double* a, const double* dadt, const double* d2adt2, int64_t n,
                         mpf_cosmology** out)
{
    if (!t || !a || !dadt || n <= 0 || n > (1 << 28) || !out) return set_err(MPF_BAD_INPUT, "mpf_cosmology_upload: bad table");
    for (int64_t i = 1; i < n; ++i)
        if (!(t[i] > t[i - 1])) return set_err(MPF_BAD_INPUT, "mpf_cosmology_upload: conformal time must increase");
    if (!has_device()) return set_err(MPF_NO_DEVICE, "mpf_cosmology_upload: no CUDA device");
    mpf_cosmology* c = new mpf_cosmology();
    cudaGetDevice(&c->device);
    c->n = (int)n;
    // search accelerator and slopes for the FP32-gather mode
    c->nlut = (int)std::min<int64_t>(4 * n, 1 << 20);
    c->t0 = t[0];
    c->lut_scale = (n > 1) ? (double)c->nlut / (t[n - 1] - t[0]) : 0.0;
    std::vector<int> lut((size_t)c->nlut + 1);
    {
        int64_t i = 0;
        for (int k = 0; k <= c->nlut; ++k) {
            const double x = c->t0 + (double)k / (c->lut_scale > 0 ? c->lut_scale : 1.0);
            while (i < n && !(x < t[i])) ++i;
            lut[(size_t)k] = (int)i;
        }
    }
    std::vector<double> sa((size_t)n, 0.0), sd((size_t)n, 0.0);
    std::vector<float2> seg((size_t)n, make_float2(0.f, 0.f));
    for (int64_t i = 0; i + 1 < n; ++i) {
        sa[(size_t)i] = (a[i + 1] - a[i]) / (t[i + 1] - t[i]);
        sd[(size_t)i] = (dadt[i + 1] - dadt[i]) / (t[i + 1] - t[i]);
        seg[(size_t)i] = make_float2((float)sd[(size_t)i], (float)(t[i + 1] - t[i]));
    }
    const size_t bytes = (size_t)n * sizeof(double);
    cudaError_t e = cudaMalloc(&c->t, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&c->a, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&c->dadt, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&c->d2adt2, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&c->slope_a, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&c->slope_dadt, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&c->lut, lut.size() * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&c->seg, seg.size() * sizeof(float2));
    if (e == cudaSuccess) e = cudaMemcpy(c->seg, seg.data(), seg.size() * sizeof(float2), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(c->t, t, bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(c->a, a, bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(c->dadt, dadt, bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = d2adt2 ? cudaMemcpy(c->d2adt2, d2adt2, bytes, cudaMemcpyHostToDevice) : cudaMemset(c->d2adt2, 0, bytes);
    if (e == cudaSuccess) e = cudaMemcpy(c->slope_a, sa.data(), bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(c->slope_dadt, sd.data(), bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(c->lut, lut.data(), lut.size() * sizeof(int), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        mpf_cosmology_destroy(c);
        return cuda_err(e, "mpf_cosmology_upload");
    }
    *out = c;
    return MPF_OK;
}

void mpf_cosmology_destroy(mpf_cosmology* c)
{
    if (!c) return;
    cudaFree(c->t);
    cudaFree(c->a);
    cudaFree(c->dadt);
    cudaFree(c->d2adt2);
    cudaFree(c->slope_a);
    cudaFree(c->slope_dadt);
    cudaFree(c->seg);
    cudaFree(c->lut);
    delete c;
}

static int gather_host(const mpf_octree* o, int kind, int exact, int64_t n, const double* xyz, void* out, size_t out_elem)
{
    if (!o || n < 0 || (n > 0 && (!xyz || !out))) return set_err(MPF_BAD_INPUT, "gather: bad argument");
    if (n == 0) return MPF_OK;
    DBuf dx, dout;
    cudaError_t e = dx.alloc((size_t)n * 3 * sizeof(double));
    if (e == cudaSuccess) e = dout.alloc((size_t)n * out_elem);
    if (e == cudaSuccess) e = cudaMemcpy(dx.p, xyz, (size_t)n * 3 * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = exact ? mpf::launch_gather_exact(o->tree, kind, (const double*)dx.p, n, dout.p, 0)
                  : mpf::launch_gather_fast(o->tree, kind, (const double*)dx.p, n, dout.p, 0);
    if (e == cudaSuccess) e = cudaMemcpy(out, dout.p, (size_t)n * out_elem, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_err(e, "gather");
    return MPF_OK;
}

int mpf_locate(const mpf_octree* o, int64_t n, const double* xyz, int64_t* cell)
{
    return gather_host(o, 0, 1, n, xyz, cell, sizeof(int64_t));
}

int mpf_interpolate(const mpf_octree* o, int order, int exact, int64_t n, const double* xyz, float* out7)
{
    if (order < 0 || order > 2) return set_err(MPF_BAD_INPUT, "mpf_interpolate: order must be 0 (NGP), 1 (CIC) or 2 (TSC)");
    // NGP copies the cell's record: no arithmetic to differ between the modes
    return (order == 0) ? gather_host(o, 3, 1, n, xyz, out7, 7 * sizeof(float))
                        : gather_host(o, order, exact, n, xyz, out7, 7 * sizeof(float));
}

int mpf_propagate_device(const mpf_octree* o, const mpf_cosmology* c, const mpf_params* p, int64_t n,
                         const double* launch_device, int64_t* steps_device, double* final_device, double* plane_device,
                         uint32_t* status_device, void* stream)
{
    mpf::PropParams P;
    if (!o || !c || !fill_params(p, P) || n < 0 || (n > 0 && (!launch_device || !steps_device || !status_device)))
        return set_err(MPF_BAD_INPUT, "mpf_propagate_device: bad argument");
    const mpf::DevCosmo C = dev_cosmo(c);
    mpf::PropOut O{(long long*)steps_device, final_device, plane_device, (unsigned*)status_device, nullptr};
    const cudaError_t e = p->exact ? mpf::launch_propagate<true>(o->tree, C, P, launch_device, n, O, (cudaStream_t)stream)
                                   : mpf::launch_propagate<false>(o->tree, C, P, launch_device, n, O, (cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_err(e, "mpf_propagate_device");
    return MPF_OK;
}

int mpf_propagate(const mpf_octree* o, const mpf_cosmology* c, const mpf_params* p, int64_t n, const double* launch,
                  int64_t* steps, double* final_rec, double* plane_rec)
{
    mpf::PropParams P;
    if (!o || !c || !fill_params(p, P) || n < 0 || (n > 0 && !launch))
        return set_err(MPF_BAD_INPUT, "mpf_propagate: bad argument");
    if (n == 0) return MPF_OK;
    cudaStream_t st = nullptr;
    cudaError_t e = host_stream(&st);
    if (e != cudaSuccess) return cuda_err(e, "mpf_propagate");
    const int np = p->nplanes;
    DBuf dl, ds, df, dp, dst;
    e = dl.alloc((size_t)n * 6 * sizeof(double));
    if (e == cudaSuccess) e = ds.alloc((size_t)n * sizeof(int64_t));
    if (e == cudaSuccess && final_rec) e = df.alloc((size_t)n * MPF_PHOTON_FIELDS * sizeof(double));
    if (e == cudaSuccess && plane_rec && np > 0) e = dp.alloc((size_t)n * np * MPF_PLANE_FIELDS * sizeof(double));
    if (e == cudaSuccess) e = dst.alloc(sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemsetAsync(dst.p, 0, sizeof(uint32_t), st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dl.p, launch, (size_t)n * 6 * sizeof(double), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_err(e, "mpf_propagate");
    int rc = mpf_propagate_device(o, c, p, n, (const double*)dl.p, (int64_t*)ds.p, (double*)df.p, (double*)dp.p,
                                  (uint32_t*)dst.p, st);
    if (rc != MPF_OK) return rc;
    uint32_t status = 0;
    e = cudaMemcpyAsync(&status, dst.p, sizeof(status), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && steps)
        e = cudaMemcpyAsync(steps, ds.p, (size_t)n * sizeof(int64_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && final_rec)
        e = cudaMemcpyAsync(final_rec, df.p, (size_t)n * MPF_PHOTON_FIELDS * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && plane_rec && np > 0)
        e = cudaMemcpyAsync(plane_rec, dp.p, (size_t)n * np * MPF_PLANE_FIELDS * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_err(e, "mpf_propagate");
    if (status & 1u) return set_err(MPF_WARN_MAX_STEPS, "mpf_propagate: a ray reached max_steps");
    return MPF_OK;
}

namespace {
// angle (rad) between a launch direction and the vector from the launch
// point to the ray's last position: atan2(|d x r|, d . r)
double deflection_of(const double* L, const double* f)
{
    const double d[3] = {L[3] - L[0], L[4] - L[1], L[5] - L[2]};
    const double r[3] = {f[2] - L[0], f[3] - L[1], f[4] - L[2]};
    const double cx = d[1] * r[2] - d[2] * r[1], cy = d[2] * r[0] - d[0] * r[2], cz = d[0] * r[1] - d[1] * r[0];
    return std::atan2(std::sqrt(cx * cx + cy * cy + cz * cz), d[0] * r[0] + d[1] * r[1] + d[2] * r[2]);
}
void lensing_of(const double* rec, double* q)
{
    const double a11 = rec[6], a12 = rec[7], a22 = rec[8];
    q[0] = 1.0 - (a11 + a22) * 0.5;
    q[1] = -0.5 * (a11 - a22);
    q[2] = -a12;
    q[3] = a11 * a22 - a12 * a12;
}
double median_of(std::vector<double>& v)
{
    if (v.empty()) return 0.0;
    const size_t h = v.size() / 2;
    std::nth_element(v.begin(), v.begin() + h, v.end());
    const double hi = v[h];
    if (v.size() % 2) return hi;
    return 0.5 * (*std::max_element(v.begin(), v.begin() + h) + hi);
}
}  // namespace

extern "C" int mpf_propagate_accuracy(const mpf_octree* o, const mpf_cosmology* c, const mpf_params* p, int64_t n,
                                      const double* launch, int64_t sample, mpf_accuracy* out)
{
    mpf::PropParams P;
    if (!o || !c || !out || !fill_params(p, P) || n <= 0 || !launch || sample <= 0)
        return set_err(MPF_BAD_INPUT, "mpf_propagate_accuracy: bad argument");
    std::memset(out, 0, sizeof(*out));
    const int64_t m = std::min(sample, n);
    const int np = p->nplanes;
    std::vector<double> L((size_t)m * 6);
    for (int64_t k = 0; k < m; ++k) {
        const int64_t src = (int64_t)(((__int128)k * n) / m);
        std::memcpy(&L[(size_t)k * 6], launch + 6 * src, 6 * sizeof(double));
    }
    std::vector<int64_t> s0((size_t)m), s1((size_t)m);
    std::vector<double> f0((size_t)m * MPF_PHOTON_FIELDS), f1((size_t)m * MPF_PHOTON_FIELDS);
    std::vector<double> q0((size_t)m * np * MPF_PLANE_FIELDS + 1), q1((size_t)m * np * MPF_PLANE_FIELDS + 1);
    mpf_params q = *p;
    q.exact = 1;
    const int rc0 = mpf_propagate(o, c, &q, m, L.data(), s0.data(), f0.data(), np ? q0.data() : nullptr);
    if (rc0 < 0) return rc0;
    q.exact = 0;
    const int rc1 = mpf_propagate(o, c, &q, m, L.data(), s1.data(), f1.data(), np ? q1.data() : nullptr);
    if (rc1 < 0) return rc1;
    out->rays = m;
    std::vector<double> dr, zr;
    dr.reserve((size_t)m);
    zr.reserve((size_t)m);
    for (int64_t k = 0; k < m; ++k) {
        const int64_t ds = s1[(size_t)k] > s0[(size_t)k] ? s1[(size_t)k] - s0[(size_t)k] : s0[(size_t)k] - s1[(size_t)k];
        if (ds) ++out->step_count_differs;
        out->max_step_diff = std::max(out->max_step_diff, ds);
        const double* a = &f0[(size_t)k * MPF_PHOTON_FIELDS];
        const double* b = &f1[(size_t)k * MPF_PHOTON_FIELDS];
        const double t0 = deflection_of(&L[(size_t)k * 6], a), t1 = deflection_of(&L[(size_t)k * 6], b);
        dr.push_back(std::fabs(t1 - t0) / std::max(std::fabs(t0), 1e-300));
        zr.push_back(std::fabs(b[19] - a[19]) / std::max(std::fabs(a[19]), 1e-300));
        for (int j = 0; j < np; ++j) {
            const double* ra = &q0[((size_t)k * np + j) * MPF_PLANE_FIELDS];
            const double* rb = &q1[((size_t)k * np + j) * MPF_PLANE_FIELDS];
            const bool va = ra[19] != 0.0, vb = rb[19] != 0.0;
            if (va != vb) ++out->surface_valid_differs;
            if (!(va && vb)) continue;
            double la[4], lb[4];
            lensing_of(ra, la);
            lensing_of(rb, lb);
            for (int t = 0; t < 4; ++t) {
                out->lensing_abs_max[t] = std::max(out->lensing_abs_max[t], std::fabs(lb[t] - la[t]));
                out->lensing_scale[t] = std::max(out->lensing_scale[t], std::fabs(la[t]));
            }
        }
    }
    out->deflection_rel_max = *std::max_element(dr.begin(), dr.end());
    out->redshift_rel_max = *std::max_element(zr.begin(), zr.end());
    out->deflection_rel_median = median_of(dr);
    out->redshift_rel_median = median_of(zr);
    return (rc0 > 0 || rc1 > 0) ? set_err(MPF_WARN_MAX_STEPS, "mpf_propagate_accuracy: a ray reached max_steps") : MPF_OK;
}

namespace {
bool catalogue_consts(const mpf_catalogue_params* p, mpf::CatConst& K, mpf::CatRotation& R)
{
    if (!p || p->nsteps == 0 || p->order < 0 || p->order > 2 || !(p->length > 0.0) || !(p->h > 0.0) ||
        !(p->mpc > 0.0) || p->max_iterations < 0 || p->max_iterations > 1000 || !(p->cat_accuracy >= 0.0))
        return false;
    K.length = p->length; K.h = p->h; K.mpc = p->mpc; K.accuracy = p->cat_accuracy;
    for (int k = 0; k < 3; ++k) K.vobs[k] = p->vobs[k];
    K.max_iterations = p->max_iterations;
    K.bundle = p->jacobian_bundle ? 1 : 0;
    K.plane_sachs = p->plane_sachs ? 1 : 0;
    K.stop_bundle = p->stop_bundle;
    K.openingmin = p->openingmin;
    K.born = p->jacobian_born ? 1 : 0;
    if (K.born && K.bundle) return false;
    if (K.bundle && (p->stop_bundle < 0 || p->stop_bundle > 5 || !(p->openingmin > 0.0) || !(p->openingmin < 1.0)))
        return false;
    if (p->rotm1)
        for (int j = 0; j < 3; ++j)
            for (int k = 0; k < 3; ++k) R.m[j][k] = p->rotm1[3 * j + k];
    return true;
}
}  // namespace

int mpf_catalogue_newton_device(const mpf_octree* o, const mpf_cosmology* c, const mpf_catalogue_params* p, int64_t n,
                                const double* sources_device, int64_t stride, double* rows_device,
                                mpf_catalogue_stats* stats, void* stream)
{
    mpf::CatConst K;
    mpf::CatRotation R;
    if (!o || !c || n < 0 || (n > 0 && (!sources_device || !rows_device)) || stride < 6 || stride > 1024)
        return set_err(MPF_BAD_INPUT, "mpf_catalogue_newton: null argument or stride < 6");
    if (o->tree.vel)
        return set_err(MPF_BAD_INPUT, "mpf_catalogue_newton: the octree carries a velocity field; the reference's "
                                      "catalogues do not run in that build (catalogues.cpp:290-293)");
    if (!catalogue_consts(p, K, R)) return set_err(MPF_BAD_INPUT, "mpf_catalogue_newton: bad parameters");
    if (n > 0x7fffffffll) return set_err(MPF_BAD_INPUT, "mpf_catalogue_newton: at most 2^31 - 1 sources per call");
    if (stats) std::memset(stats, 0, sizeof(*stats));
    if (n == 0) return MPF_OK;
    const mpf::DevCosmo C = dev_cosmo(c);
    mpf::CatRunStats st;
    unsigned status = 0;
    const cudaError_t e = mpf::catalogue_newton(o->tree, C, K, p->rotm1 ? &R : nullptr, p->exact != 0, p->order, p->nsteps,
                                                n, sources_device, (int)stride, rows_device, &st, &status,
                                                (cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_err(e, "mpf_catalogue_newton");
    if (stats) {
        stats->rays = st.rays;
        stats->photon_steps = st.photon_steps;
        stats->photon_steps_jacobian = st.photon_steps_jacobian;
        stats->iterations = st.iterations;
        stats->kernel_launches = st.launches;
    }
    if (status & mpf::kCatQueueError)
        return set_err(MPF_DEVICE_TIMEOUT, std::string("mpf_catalogue_newton: the device work queue lost a source (a bounded "
                                                       "wait ran out): ") + mpf::catalogue_queue_message());
    if (status & 1u) return set_err(MPF_WARN_MAX_STEPS, "mpf_catalogue_newton: a ray reached max_steps");
    return MPF_OK;
}

int mpf_catalogue_newton(const mpf_octree* o, const mpf_cosmology* c, const mpf_catalogue_params* p, int64_t n,
                         const double* sources, int64_t stride, double* rows, mpf_catalogue_stats* stats)
{
    mpf::CatConst K;
    mpf::CatRotation R;
    if (!o || !c || n < 0 || (n > 0 && (!sources || !rows)) || stride < 6 || stride > 1024)
        return set_err(MPF_BAD_INPUT, "mpf_catalogue_newton: null argument or stride < 6");
    if (o->tree.vel)
        return set_err(MPF_BAD_INPUT, "mpf_catalogue_newton: the octree carries a velocity field; the reference's "
                                      "catalogues do not run in that build (catalogues.cpp:290-293)");
    if (!catalogue_consts(p, K, R)) return set_err(MPF_BAD_INPUT, "mpf_catalogue_newton: bad parameters");
    if (stats) std::memset(stats, 0, sizeof(*stats));
    if (n == 0) return MPF_OK;
    DBuf dsrc, drows;
    cudaError_t e = dsrc.alloc((size_t)n * (size_t)stride * sizeof(double));
    if (e == cudaSuccess) e = drows.alloc((size_t)n * MPF_CATALOGUE_FIELDS * sizeof(double));
    if (e == cudaSuccess) e = cudaMemcpy(dsrc.p, sources, (size_t)n * (size_t)stride * sizeof(double), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_err(e, "mpf_catalogue_newton");
    const int rc = mpf_catalogue_newton_device(o, c, p, n, (const double*)dsrc.p, stride, (double*)drows.p, stats, nullptr);
    if (rc < 0) return rc;
    e = cudaMemcpy(rows, drows.p, (size_t)n * MPF_CATALOGUE_FIELDS * sizeof(double), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_err(e, "mpf_catalogue_newton");
    return rc;
}

namespace {
int hmaps_fill_impl(const mpf_octree* o, const mpf_cosmology* c, const mpf_params* p, int64_t nside, int64_t npix,
                    const int64_t* pixels, int ncomp, const int* components, const double* homogeneous, float* maps,
                    int bundle, int plane_sachs, int stop_bundle, double openingmin)
{
    mpf::PropParams P;
    if (!o || !c || !fill_params(p, P) || npix < 0 || (npix > 0 && (!pixels || !maps)) || nside < 1 ||
        nside > (1ll << 29) || ncomp < 1 || ncomp > MPF_MAX_MAP_COMPONENTS || !components || !homogeneous)
        return set_err(MPF_BAD_INPUT, "mpf_hmaps_fill: bad argument");
    if (p->nplanes < 1) return set_err(MPF_BAD_INPUT, "mpf_hmaps_fill: at least one surface (p->planes) is needed");
    if (p->stop == MPF_STOP_PLANE) return set_err(MPF_BAD_INPUT, "mpf_hmaps_fill: stop_ray 'plane' has no map surfaces");
    mpf::MapSpec M;
    std::memset(&M, 0, sizeof(M));
    M.ncomp = ncomp;
    for (int q = 0; q < ncomp; ++q) {
        const int k = components[q];
        if (k < 0 || k > 13) return set_err(MPF_BAD_INPUT, "mpf_hmaps_fill: unknown map component");
        M.comp[q] = k;
        M.nmaps += (k == MPF_MAP_LENSING) ? (bundle ? 5 : 4) : (k == MPF_MAP_LENSING_BORN) ? 4 : (k == MPF_MAP_DEFLECTION) ? 2 : 1;
        if (k == MPF_MAP_LENSING_BORN) M.born = 1;
    }
    // lensing_born alone: no ray is traced through the field (hmaps.h:594, 604-605)
    M.only_born = (ncomp == 1 && components[0] == MPF_MAP_LENSING_BORN) ? 1 : 0;
    if (bundle) {
        // Lensing::dbetadtheta knows lambda, r, redshift, a, t and plane (lensing.h:198-296)
        if (stop_bundle < 0 || stop_bundle > 5 || !(openingmin > 0.0) || !(openingmin < 1.0))
            return set_err(MPF_BAD_INPUT, "mpf_hmaps_fill_bundle: stop_bundle must be redshift, r, lambda, t, a or plane, "
                                          "and 0 < openingmin < 1 radian");
        M.bundle = 1;
        M.plane_sachs = plane_sachs ? 1 : 0;
        M.stop_bundle = stop_bundle;
        M.openingmin = openingmin;
    }
    for (int iz = 0; iz < p->nplanes; ++iz)
        for (int k = 0; k < 5; ++k) M.homogeneous[iz][k] = homogeneous[5 * iz + k];
    const long long npixall = 12ll * nside * nside;
    for (int64_t i = 0; i < npix; ++i)
        if (pixels[i] < 0 || pixels[i] >= npixall) return set_err(MPF_BAD_INPUT, "mpf_hmaps_fill: pixel id out of range");
    P.jacobian = 1;
    if (npix == 0) return MPF_OK;
    const mpf::DevCosmo C = dev_cosmo(c);
    const size_t map_bytes = (size_t)M.nmaps * (size_t)p->nplanes * (size_t)npix * sizeof(float);
    DBuf dpix, dmaps;
    cudaError_t e = dpix.alloc((size_t)npix * sizeof(int64_t));
    if (e == cudaSuccess) e = dmaps.alloc(map_bytes);
    if (e == cudaSuccess) e = cudaMemcpy(dpix.p, pixels, (size_t)npix * sizeof(int64_t), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_err(e, "mpf_hmaps_fill");
    unsigned status = 0;
    e = mpf::hmaps_fill(o->tree, C, P, p->exact != 0, nside, npix, (const long long*)dpix.p, M, (float*)dmaps.p,
                        1ll << 22, &status, nullptr);
    if (e == cudaSuccess) e = cudaMemcpy(maps, dmaps.p, map_bytes, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_err(e, "mpf_hmaps_fill");
    if (status & 1u) return set_err(MPF_WARN_MAX_STEPS, "mpf_hmaps_fill: a ray reached max_steps");
    return MPF_OK;
}
}  // namespace

int mpf_hmaps_fill(const mpf_octree* o, const mpf_cosmology* c, const mpf_params* p, int64_t nside, int64_t npix,
                   const int64_t* pixels, int ncomp, const int* components, const double* homogeneous, float* maps)
{
    return hmaps_fill_impl(o, c, p, nside, npix, pixels, ncomp, components, homogeneous, maps, 0, 0, 0, 0.0);
}

int mpf_hmaps_fill_bundle(const mpf_octree* o, const mpf_cosmology* c, const mpf_params* p, int64_t nside, int64_t npix,
                          const int64_t* pixels, int ncomp, const int* components, const double* homogeneous,
                          int plane_sachs, int stop_bundle, double openingmin, float* maps)
{
    return hmaps_fill_impl(o, c, p, nside, npix, pixels, ncomp, components, homogeneous, maps, 1, plane_sachs,
                           stop_bundle, openingmin);
}

int mpf_autotune_info(const mpf_octree* o, int kind, int order, int* threads_per_block, int* claim_depth, double* rates)
{
    if (!o || !threads_per_block || !claim_depth || (kind != 0 && kind != 1) || (order != 1 && order != 2))
        return set_err(MPF_BAD_INPUT, "mpf_autotune_info: bad argument");
    int dev = 0;
    const cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_err(e, "mpf_autotune_info");
    *threads_per_block = 0;
    *claim_depth = 0;
    double r[4] = {0, 0, 0, 0};
    int tpb = 0, depth = 1;
    bool ok = (kind == 0) ? mpf::tuned_shape(dev, o->tree, mpf::plain_fast_mode(order, o->tree.vel != nullptr), &tpb, &depth, r)
                          : mpf::catalogue_tuned_shape(dev, o->tree, order, &tpb, r);
    if (ok) {
        *threads_per_block = tpb;
        *claim_depth = depth;
    }
    if (rates)
        for (int k = 0; k < 4; ++k) rates[k] = r[k];
    return MPF_OK;
}

int mpf_pix2vec_ring(int64_t nside, int64_t n, const int64_t* pixels, double* vec)
{
    if (nside < 1 || nside > (1ll << 29) || n < 0 || (n > 0 && (!pixels || !vec)))
        return set_err(MPF_BAD_INPUT, "mpf_pix2vec_ring: bad argument");
    for (int64_t i = 0; i < n; ++i)
        if (pixels[i] < 0 || pixels[i] >= 12ll * nside * nside) return set_err(MPF_BAD_INPUT, "mpf_pix2vec_ring: pixel id out of range");
    if (n == 0) return MPF_OK;
    if (!has_device()) return set_err(MPF_NO_DEVICE, "mpf_pix2vec_ring: no CUDA device");
    DBuf dpix, dl;
    cudaError_t e = dpix.alloc((size_t)n * sizeof(int64_t));
    if (e == cudaSuccess) e = dl.alloc((size_t)n * 6 * sizeof(double));
    if (e == cudaSuccess) e = cudaMemcpy(dpix.p, pixels, (size_t)n * sizeof(int64_t), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = mpf::pix2vec_device(nside, n, (const long long*)dpix.p, (double*)dl.p, nullptr);
    std::vector<double> L;
    if (e == cudaSuccess) {
        L.resize((size_t)n * 6);
        e = cudaMemcpy(L.data(), dl.p, (size_t)n * 6 * sizeof(double), cudaMemcpyDeviceToHost);
    }
    if (e != cudaSuccess) return cuda_err(e, "mpf_pix2vec_ring");
    for (int64_t i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k) vec[3 * i + k] = L[6 * i + 3 + k];
    return MPF_OK;
}

}  // extern "C"
