// femsolver.cu -- the FEMSolver_ handle behind the C ABI (include/pfg.h).
//
// Mirrors the state of plantFEM's FEMSolver_ (FEMSolverClass.f90:13-164):
// one domain (mesh), the working CRS matrix (CRS_val / CRS_Index_*), CRS_RHS,
// the fix list (fix_lin_exists / fix_lin_exists_values), and the named matrix
// stack of keepThisMatrixAs.  All of it lives on the device; host arrays are
// copied in at set*/fix and out at solve/eig/getCRS, like the reference's
// value-semantics setters.
#include <algorithm>
#include <numeric>
#include <chrono>
#include <cmath>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "assembly.cuh"
#include "batch.cuh"
#include "ilu.cuh"

namespace pfg {

static thread_local std::string g_last_error;
void set_last_error(const std::string &msg) { g_last_error = msg; }

}  // namespace pfg

using namespace pfg;

struct pfg_solver {
    std::mutex mu;
    cudaStream_t st = nullptr;
    int device = 0;
    DevMesh mesh;
    bool have_mesh = false;
    DevMatrix K;
    bool have_crs = false;
    DevBuf<double> rhs;
    std::vector<uint8_t> fixed_h;
    std::vector<double> fixval_h;
    bool have_fix = false;
    DevBuf<uint8_t> fixed_d;
    DevBuf<double> fixval_d;
    // buffered setMatrix / setVector calls (0-based element ids)
    std::vector<int> pend_mat_ids;
    std::vector<double> pend_mats;
    std::vector<int> pend_vec_ids;
    std::vector<double> pend_vecs;
    Krylov kry;
    DevBuf<double> x;
    // keepThisMatrixAs stack (FEMSolverClass.f90:1544-1604), at most 10 names
    std::vector<std::pair<std::string, DevMatrix>> stack;
    std::vector<int> fix_eig_ids;  // 1-based, unique, sorted (fix_eig, :1607-1628)
    // linear Newmark-beta time stepping (pfg_newmark_*): parameters and state
    struct Newmark {
        bool ready = false;
        double dt = 0, beta = 0, gamma = 0, ray_alpha = 0, ray_beta = 0;
        DevBuf<double> u, v, a, base, wM, wK, rhs, tmp, x;
    } nm;

    int64_t ndof() const { return K.ndof(); }
};

namespace {

void need(bool c, int code, const char *msg)
{
    if (!c) throw Error(code, msg);
}

void flush_pending(pfg_solver *h)
{
    if (!h->pend_mat_ids.empty()) {
        const int64_t cnt = (int64_t)h->pend_mat_ids.size();
        DevBuf<int> ids((size_t)cnt);
        DevBuf<double> mats((size_t)cnt * 576);
        PFG_CUDA(cudaMemcpyAsync(ids.p, h->pend_mat_ids.data(), cnt * sizeof(int), cudaMemcpyHostToDevice, h->st));
        PFG_CUDA(cudaMemcpyAsync(mats.p, h->pend_mats.data(), cnt * 576 * sizeof(double), cudaMemcpyHostToDevice,
                                 h->st));
        scatter_element_matrices(h->mesh, h->K, cnt, ids.p, mats.p, h->st);
        h->pend_mat_ids.clear();
        h->pend_mats.clear();
    }
    if (!h->pend_vec_ids.empty()) {
        const int64_t cnt = (int64_t)h->pend_vec_ids.size();
        DevBuf<int> ids((size_t)cnt);
        DevBuf<double> vecs((size_t)cnt * 24);
        PFG_CUDA(cudaMemcpyAsync(ids.p, h->pend_vec_ids.data(), cnt * sizeof(int), cudaMemcpyHostToDevice, h->st));
        PFG_CUDA(cudaMemcpyAsync(vecs.p, h->pend_vecs.data(), cnt * 24 * sizeof(double), cudaMemcpyHostToDevice,
                                 h->st));
        scatter_element_vectors(h->mesh, h->rhs.p, cnt, ids.p, vecs.p, h->st);
        h->pend_vec_ids.clear();
        h->pend_vecs.clear();
    }
}

void reset_system(pfg_solver *h)
{
    const int64_t n = h->ndof();
    h->rhs.alloc((size_t)std::max<int64_t>(n, 1));
    PFG_CUDA(cudaMemsetAsync(h->rhs.p, 0, n * sizeof(double), h->st));
    h->fixed_h.assign((size_t)n, 0);
    h->fixval_h.assign((size_t)n, 0.0);
    h->have_fix = false;
    h->have_crs = true;
}

// setCRS(DOF): pattern from the mesh
void set_crs_from_mesh(pfg_solver *h)
{
    need(h->have_mesh, PFG_E_STATE, "setCRS before setDomain: no mesh");
    build_pattern(h->mesh, h->K, h->st);
    reset_system(h);
}

void ensure_crs(pfg_solver *h)
{
    if (!h->have_crs) set_crs_from_mesh(h);  // setValue calls setCRS itself (FEMSolverClass.f90:1015-1017)
}

KConfig to_config(const pfg_solve_opts *o)
{
    pfg_solve_opts d;
    pfg_solve_opts_default(&d);
    if (!o) o = &d;
    KConfig c;
    c.algorithm = o->algorithm;
    c.precision = o->precision;
    c.precond = o->precond;
    c.stop_rule = o->stop_rule;
    c.itrmax = o->itrmax;
    c.er0 = o->er0;
    c.relative_er = o->relative_er;
    c.reliable_delta = o->reliable_delta;
    c.graph_chunk = o->graph_chunk;
    c.debug = o->debug;
    c.fuse = o->update_mode == 1 ? 1 : (o->update_mode == 2 ? 0 : -1);
    c.storage = o->storage;
    return c;
}

void fill_info(pfg_info *info, const SolveResult &r, int precision)
{
    if (!info) return;
    info->status = r.status;
    info->iterations = r.iterations;
    info->replacements = r.replacements;
    info->kernel_launches = r.launches;
    (void)precision;
    info->rel_residual = r.rel_residual;
    info->iter_residual = r.iter_residual;
    info->solve_ms = r.ms;
    info->fallback = r.fallback;
}

int solve_status(const SolveResult &r)
{
    if (r.status == PFG_E_BREAKDOWN || r.status == PFG_E_NONFINITE) {
        set_last_error(r.status == PFG_E_BREAKDOWN ? "Krylov breakdown (Bicgstab devide by zero)"
                                                   : "non-finite value in a Krylov scalar");
        return r.status;
    }
    if (r.status == PFG_W_NOT_CONVERGED) set_last_error("not converged within itrmax");
    return r.status;
}

void apply_fix_device(pfg_solver *h)
{
    if (!h->have_fix) return;
    const int64_t n = h->ndof();
    h->fixed_d.ensure((size_t)n);
    h->fixval_d.ensure((size_t)n);
    PFG_CUDA(cudaMemcpyAsync(h->fixed_d.p, h->fixed_h.data(), n, cudaMemcpyHostToDevice, h->st));
    PFG_CUDA(cudaMemcpyAsync(h->fixval_d.p, h->fixval_h.data(), n * sizeof(double), cudaMemcpyHostToDevice, h->st));
    apply_dirichlet(h->K, h->rhs.p, h->fixed_d.p, h->fixval_d.p, h->st);
}

}  // namespace

extern "C" {

void pfg_solve_opts_default(pfg_solve_opts *o)
{
    if (!o) return;
    memset(o, 0, sizeof(*o));
    o->algorithm = PFG_ALG_BICGSTAB;
    o->precision = PFG_PREC_FP64;
    o->precond = PFG_PC_NONE;
    o->stop_rule = PFG_STOP_REFERENCE;
    o->itrmax = 100000;
    o->graph_chunk = 32;
    o->er0 = 1.0e-10;
    o->relative_er = 1.0e-10;
    o->reliable_delta = 0.1;
    o->debug = 0;
}

const char *pfg_last_error(void) { return g_last_error.c_str(); }
const char *pfg_version(void) { return "plantfem_gb300 0.1 (sm_103a)"; }

int pfg_create(pfg_solver **out)
{
    return guard([&] {
        need(out != nullptr, PFG_E_ARG, "NULL handle pointer");
        pfg_solver *h = new pfg_solver();
        try {
            PFG_CUDA(cudaGetDevice(&h->device));
            PFG_CUDA(cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking));
        } catch (...) {
            delete h;
            throw;
        }
        *out = h;
    });
}

int pfg_destroy(pfg_solver *h)
{
    return guard([&] {
        if (!h) return;
        {
            std::lock_guard<std::mutex> lk(h->mu);
            cudaStreamSynchronize(h->st);
        }
        cudaStream_t st = h->st;
        delete h;
        if (st) cudaStreamDestroy(st);
    });
}

int pfg_set_mesh(pfg_solver *h, int64_t nn, const double *nodcoord, int64_t ne, int32_t nne, const int32_t *elemnod)
{
    return guard([&] {
        need(h && nodcoord && elemnod, PFG_E_ARG, "NULL argument");
        need(nne == 8, PFG_E_UNSUPPORTED, "only 8-node hexahedra are supported");
        need(nn > 0 && ne > 0 && nn < INT32_MAX, PFG_E_ARG, "bad mesh size");
        std::lock_guard<std::mutex> lk(h->mu);
        DevMesh &m = h->mesh;
        m.nn = nn;
        m.ne = ne;
        m.conn_host.resize((size_t)ne * 8);
        for (int64_t i = 0; i < ne * 8; ++i) {
            const int32_t v = elemnod[i];
            need(v >= 1 && v <= nn, PFG_E_ARG, "ElemNod entry out of range 1..nn");
            m.conn_host[(size_t)i] = v - 1;
        }
        for (int64_t i = 0; i < nn * 3; ++i) need(std::isfinite(nodcoord[i]), PFG_E_NONFINITE, "non-finite NodCoord");
        m.xyz.alloc((size_t)nn * 3);
        m.conn.alloc((size_t)ne * 8);
        PFG_CUDA(cudaMemcpyAsync(m.xyz.p, nodcoord, nn * 3 * sizeof(double), cudaMemcpyHostToDevice, h->st));
        PFG_CUDA(cudaMemcpyAsync(m.conn.p, m.conn_host.data(), ne * 8 * sizeof(int), cudaMemcpyHostToDevice, h->st));
        color_elements(m, h->st);
        h->have_mesh = true;
        h->have_crs = false;
    });
}

int pfg_set_crs(pfg_solver *h, int32_t dof)
{
    return guard([&] {
        need(h != nullptr, PFG_E_ARG, "NULL handle");
        need(dof == 3, PFG_E_UNSUPPORTED, "setCRS: only DOF=3 (linear elasticity) is supported");
        std::lock_guard<std::mutex> lk(h->mu);
        set_crs_from_mesh(h);
    });
}

int pfg_set_crs_arrays(pfg_solver *h, int64_t n, const int64_t *row_ptr, const int32_t *col_idx, const double *val)
{
    return guard([&] {
        need(h && row_ptr && col_idx && val && n > 0, PFG_E_ARG, "bad CRS arguments");
        need(row_ptr[0] == 1, PFG_E_ARG, "row_ptr(1) must be 1");
        const int64_t nnz = row_ptr[n] - 1;
        need(nnz >= 0, PFG_E_ARG, "row_ptr(n+1) < 1");
        std::lock_guard<std::mutex> lk(h->mu);
        DevBuf<int64_t> rp((size_t)n + 1);
        DevBuf<int32_t> ci((size_t)std::max<int64_t>(nnz, 1));
        DevBuf<double> v((size_t)std::max<int64_t>(nnz, 1));
        PFG_CUDA(cudaMemcpyAsync(rp.p, row_ptr, (n + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, h->st));
        PFG_CUDA(cudaMemcpyAsync(ci.p, col_idx, nnz * sizeof(int32_t), cudaMemcpyHostToDevice, h->st));
        PFG_CUDA(cudaMemcpyAsync(v.p, val, nnz * sizeof(double), cudaMemcpyHostToDevice, h->st));
        import_crs(n, nnz, rp.p, ci.p, v.p, h->K, h->st);
        const bool keep_rhs = h->rhs.n >= (size_t)n && h->have_crs && h->ndof() == n;
        if (!keep_rhs) reset_system(h);
        h->have_crs = true;
        PFG_CUDA(cudaStreamSynchronize(h->st));
    });
}

int pfg_get_crs_size(pfg_solver *h, int64_t *n, int64_t *nnz)
{
    return guard([&] {
        need(h != nullptr, PFG_E_ARG, "NULL handle");
        std::lock_guard<std::mutex> lk(h->mu);
        need(h->have_crs, PFG_E_STATE, "no CRS matrix");
        if (n) *n = h->ndof();
        if (nnz) *nnz = h->K.nnzb * h->K.bs * h->K.bs;
    });
}

int pfg_get_crs(pfg_solver *h, int64_t *row_ptr, int32_t *col_idx, double *val)
{
    return guard([&] {
        need(h != nullptr, PFG_E_ARG, "NULL handle");
        std::lock_guard<std::mutex> lk(h->mu);
        need(h->have_crs, PFG_E_STATE, "no CRS matrix");
        flush_pending(h);
        const int64_t n = h->ndof(), nnz = h->K.nnzb * h->K.bs * h->K.bs;
        DevBuf<int64_t> rp(row_ptr ? (size_t)n + 1 : 0);
        DevBuf<int32_t> ci(col_idx ? (size_t)std::max<int64_t>(nnz, 1) : 0);
        DevBuf<double> v(val ? (size_t)std::max<int64_t>(nnz, 1) : 0);
        export_crs(h->K, rp.p, ci.p, v.p, h->st);
        if (row_ptr) PFG_CUDA(cudaMemcpyAsync(row_ptr, rp.p, (n + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost, h->st));
        if (col_idx) PFG_CUDA(cudaMemcpyAsync(col_idx, ci.p, nnz * sizeof(int32_t), cudaMemcpyDeviceToHost, h->st));
        if (val) PFG_CUDA(cudaMemcpyAsync(val, v.p, nnz * sizeof(double), cudaMemcpyDeviceToHost, h->st));
        PFG_CUDA(cudaStreamSynchronize(h->st));
    });
}

int pfg_set_rhs(pfg_solver *h, int64_t n, const double *rhs)
{
    return guard([&] {
        need(h && rhs, PFG_E_ARG, "NULL argument");
        std::lock_guard<std::mutex> lk(h->mu);
        ensure_crs(h);
        need(n == h->ndof(), PFG_E_ARG, "setRHS: size differs from the CRS matrix");
        PFG_CUDA(cudaMemcpyAsync(h->rhs.p, rhs, n * sizeof(double), cudaMemcpyHostToDevice, h->st));
        PFG_CUDA(cudaStreamSynchronize(h->st));
    });
}

int pfg_get_rhs(pfg_solver *h, int64_t n, double *rhs)
{
    return guard([&] {
        need(h && rhs, PFG_E_ARG, "NULL argument");
        std::lock_guard<std::mutex> lk(h->mu);
        need(h->have_crs && n == h->ndof(), PFG_E_ARG, "size differs from the CRS matrix");
        flush_pending(h);
        PFG_CUDA(cudaMemcpyAsync(rhs, h->rhs.p, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
        PFG_CUDA(cudaStreamSynchronize(h->st));
    });
}

int pfg_set_matrix(pfg_solver *h, int32_t domain_id, int32_t element_id, int32_t dof, const double *matrix)
{
    if (domain_id != 1 || dof != 3) {
        set_last_error("setMatrix: DomainID must be 1 and DOF 3");
        return PFG_E_UNSUPPORTED;
    }
    return pfg_set_matrices(h, 1, &element_id, matrix);
}

int pfg_set_matrices(pfg_solver *h, int64_t count, const int32_t *element_ids, const double *matrices)
{
    return guard([&] {
        need(h && element_ids && matrices && count >= 0, PFG_E_ARG, "NULL argument");
        std::lock_guard<std::mutex> lk(h->mu);
        need(h->have_mesh, PFG_E_STATE, "setMatrix before setDomain");
        ensure_crs(h);
        need(h->K.bs == 3, PFG_E_STATE, "setMatrix needs the mesh pattern (setCRS(DOF=3))");
        for (int64_t i = 0; i < count; ++i) {
            need(element_ids[i] >= 1 && element_ids[i] <= h->mesh.ne, PFG_E_ARG, "ElementID out of range");
            h->pend_mat_ids.push_back(element_ids[i] - 1);
        }
        h->pend_mats.insert(h->pend_mats.end(), matrices, matrices + count * 576);
        if (h->pend_mat_ids.size() >= 65536) flush_pending(h);
    });
}

int pfg_set_vector(pfg_solver *h, int32_t domain_id, int32_t element_id, int32_t dof, const double *vector)
{
    return guard([&] {
        need(h && vector, PFG_E_ARG, "NULL argument");
        need(domain_id == 1 && dof == 3, PFG_E_UNSUPPORTED, "setVector: DomainID must be 1 and DOF 3");
        std::lock_guard<std::mutex> lk(h->mu);
        need(h->have_mesh, PFG_E_STATE, "setVector before setDomain");
        ensure_crs(h);
        need(element_id >= 1 && element_id <= h->mesh.ne, PFG_E_ARG, "ElementID out of range");
        h->pend_vec_ids.push_back(element_id - 1);
        h->pend_vecs.insert(h->pend_vecs.end(), vector, vector + 24);
        if (h->pend_vec_ids.size() >= 65536) flush_pending(h);
    });
}

static void upload_prop(pfg_solver *h, int64_t n_prop, const double *p, DevBuf<double> &d, const char *name)
{
    need(p != nullptr, PFG_E_ARG, "NULL property array");
    need(n_prop == 1 || n_prop == h->mesh.ne, PFG_E_ARG,
         (std::string("size of ") + name + " should be 1 or number_of_element").c_str());
    for (int64_t i = 0; i < n_prop; ++i) need(std::isfinite(p[i]), PFG_E_NONFINITE, "non-finite material property");
    d.alloc((size_t)n_prop);
    PFG_CUDA(cudaMemcpyAsync(d.p, p, n_prop * sizeof(double), cudaMemcpyHostToDevice, h->st));
}

int pfg_assemble_stiffness(pfg_solver *h, int64_t n_prop, const double *E, const double *nu)
{
    return guard([&] {
        need(h != nullptr, PFG_E_ARG, "NULL handle");
        std::lock_guard<std::mutex> lk(h->mu);
        need(h->have_mesh, PFG_E_STATE, "assemble before setDomain");
        ensure_crs(h);
        flush_pending(h);
        DevBuf<double> dE, dnu;
        upload_prop(h, n_prop, E, dE, "E");
        upload_prop(h, n_prop, nu, dnu, "v");
        assemble_elements(h->mesh, h->K, 0, dE.p, dnu.p, n_prop == 1, h->st);
    });
}

int pfg_assemble_mass(pfg_solver *h, int64_t n_prop, const double *rho, int32_t lumped)
{
    return guard([&] {
        need(h != nullptr, PFG_E_ARG, "NULL handle");
        std::lock_guard<std::mutex> lk(h->mu);
        need(h->have_mesh, PFG_E_STATE, "assemble before setDomain");
        ensure_crs(h);
        flush_pending(h);
        DevBuf<double> dr;
        upload_prop(h, n_prop, rho, dr, "Density");
        assemble_elements(h->mesh, h->K, lumped ? 2 : 1, dr.p, nullptr, n_prop == 1, h->st);
    });
}

int pfg_assemble_body_force(pfg_solver *h, int64_t n_prop, const double *rho, const double accel[3])
{
    return guard([&] {
        need(h && accel, PFG_E_ARG, "NULL argument");
        std::lock_guard<std::mutex> lk(h->mu);
        need(h->have_mesh, PFG_E_STATE, "assemble before setDomain");
        ensure_crs(h);
        flush_pending(h);
        DevBuf<double> dr;
        upload_prop(h, n_prop, rho, dr, "Density");
        assemble_body_force(h->mesh, h->rhs.p, dr.p, n_prop == 1, accel, h->st);
    });
}

int pfg_zeros(pfg_solver *h)
{
    return guard([&] {
        need(h != nullptr, PFG_E_ARG, "NULL handle");
        std::lock_guard<std::mutex> lk(h->mu);
        need(h->have_crs, PFG_E_STATE, "zeros before setCRS");
        h->pend_mat_ids.clear();
        h->pend_mats.clear();
        h->pend_vec_ids.clear();
        h->pend_vecs.clear();
        const int64_t nv = h->K.nnzb * h->K.bs * h->K.bs;
        PFG_CUDA(cudaMemsetAsync(h->K.v64.p, 0, nv * sizeof(double), h->st));
        PFG_CUDA(cudaMemsetAsync(h->rhs.p, 0, h->ndof() * sizeof(double), h->st));
        h->K.values_changed();
        PFG_CUDA(cudaStreamSynchronize(h->st));
    });
}

int pfg_fix(pfg_solver *h, int64_t n, const int32_t *ids, const double *values, double value)
{
    return guard([&] {
        need(h && (ids || n == 0), PFG_E_ARG, "NULL argument");
        std::lock_guard<std::mutex> lk(h->mu);
        ensure_crs(h);
        const int64_t N = h->ndof();
        for (int64_t i = 0; i < n; ++i) {
            const int64_t id = ids[i];
            if (id < 1 || id > N) continue;  // FEMSolverClass.f90:1106-1109
            h->fixed_h[(size_t)id - 1] = 1;
            h->fixval_h[(size_t)id - 1] = values ? values[i] : value;
        }
        h->have_fix = true;
    });
}

int pfg_solve(pfg_solver *h, const pfg_solve_opts *opts, const double *x0, double *x_out, pfg_info *info)
{
    SolveResult res;
    const int rc = guard([&] {
        need(h && x_out, PFG_E_ARG, "NULL argument");
        std::lock_guard<std::mutex> lk(h->mu);
        need(h->have_crs, PFG_E_STATE, "solve before setCRS");
        flush_pending(h);
        const int64_t n = h->ndof();
        apply_fix_device(h);
        h->x.ensure((size_t)n);
        if (x0)
            PFG_CUDA(cudaMemcpyAsync(h->x.p, x0, n * sizeof(double), cudaMemcpyHostToDevice, h->st));
        else
            PFG_CUDA(cudaMemsetAsync(h->x.p, 0, n * sizeof(double), h->st));
        const KConfig cfg = to_config(opts);
        res = h->kry.solve(h->K, h->rhs.p, h->x.p, cfg, h->st);
        if (h->have_fix) restore_fixed(n, h->x.p, h->fixed_d.p, h->fixval_d.p, h->st);
        PFG_CUDA(cudaMemcpyAsync(x_out, h->x.p, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
        PFG_CUDA(cudaStreamSynchronize(h->st));
        fill_info(info, res, cfg.precision);
    });
    if (rc != PFG_OK) return rc;
    return solve_status(res);
}

int pfg_dev_spmv(pfg_solver *h, const double *d_x, double *d_y, void *stream)
{
    return guard([&] {
        need(h && d_x && d_y, PFG_E_ARG, "NULL argument");
        std::lock_guard<std::mutex> lk(h->mu);
        need(h->have_crs, PFG_E_STATE, "no CRS matrix");
        flush_pending(h);
        cudaStream_t st = stream ? (cudaStream_t)stream : h->st;
        if (st != h->st) PFG_CUDA(cudaStreamSynchronize(h->st));
        Krylov::spmv64_sliced(h->K, d_x, d_y, st);
        if (!stream) PFG_CUDA(cudaStreamSynchronize(st));  // own stream: done on return
    });
}

int pfg_dev_solve(pfg_solver *h, const pfg_solve_opts *opts, const double *d_b, double *d_x, pfg_info *info,
                  void *stream)
{
    SolveResult res;
    const int rc = guard([&] {
        need(h && d_b && d_x, PFG_E_ARG, "NULL argument");
        std::lock_guard<std::mutex> lk(h->mu);
        need(h->have_crs, PFG_E_STATE, "no CRS matrix");
        flush_pending(h);
        cudaStream_t st = stream ? (cudaStream_t)stream : h->st;
        if (st != h->st) PFG_CUDA(cudaStreamSynchronize(h->st));
        const KConfig cfg = to_config(opts);
        res = h->kry.solve(h->K, d_b, d_x, cfg, st);
        fill_info(info, res, cfg.precision);
    });
    if (rc != PFG_OK) return rc;
    return solve_status(res);
}

// ------------------------------------------------------ reference plug-ins
}  // extern "C"

namespace {

template <typename T>
int crs_spmv_host(const T *val, const int64_t *row_ptr, const int32_t *col_idx, const T *old_vector, T *new_vector,
                  size_t n, size_t col_size)
{
    return guard([&] {
        need(val && row_ptr && col_idx && old_vector && new_vector, PFG_E_ARG, "NULL argument");
        if (n == 0) return;
        need(row_ptr[0] == 1, PFG_E_ARG, "row_ptr(1) must be 1");
        const int64_t nnz = row_ptr[n] - 1;
        need(nnz >= 0 && (size_t)nnz <= col_size, PFG_E_ARG, "row_ptr(n+1)-1 exceeds col_size");
        cudaStream_t st;
        PFG_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        struct StreamGuard {
            cudaStream_t s;
            ~StreamGuard() { cudaStreamDestroy(s); }
        } sg{st};
        DevBuf<int64_t> rp(n + 1);
        DevBuf<int32_t> ci((size_t)std::max<int64_t>(nnz, 1));
        DevBuf<T> x(n), y(n);
        PFG_CUDA(cudaMemcpyAsync(rp.p, row_ptr, (n + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, st));
        PFG_CUDA(cudaMemcpyAsync(ci.p, col_idx, nnz * sizeof(int32_t), cudaMemcpyHostToDevice, st));
        PFG_CUDA(cudaMemcpyAsync(x.p, old_vector, n * sizeof(T), cudaMemcpyHostToDevice, st));
        // Scalar rows (1x1 blocks, one warp per row): the reference's operator
        // exactly, whatever its structure.
        DevMatrix A;
        import_crs((int64_t)n, nnz, rp.p, ci.p, nullptr, A, st, /*allow_blocks=*/false);
        if (sizeof(T) == 8) {
            PFG_CUDA(cudaMemcpyAsync(A.v64.p, val, nnz * sizeof(double), cudaMemcpyHostToDevice, st));
            Krylov::spmv64(A, (const double *)x.p, (double *)y.p, st);
        } else {
            A.v32.alloc((size_t)std::max<int64_t>(nnz, 1));
            PFG_CUDA(cudaMemcpyAsync(A.v32.p, val, nnz * sizeof(float), cudaMemcpyHostToDevice, st));
            A.v32_valid = true;
            Krylov::spmv32(A, (const float *)x.p, (float *)y.p, st);
        }
        std::vector<T> hy(n);
        PFG_CUDA(cudaMemcpyAsync(hy.data(), y.p, n * sizeof(T), cudaMemcpyDeviceToHost, st));
        PFG_CUDA(cudaStreamSynchronize(st));
        // SparseClass-c.c:61-63 accumulates into new_vector
        for (size_t i = 0; i < n; ++i) new_vector[i] = new_vector[i] + hy[i];
    });
}

}  // namespace

extern "C" {

int pfg_crs_spmv_real64(const double *val, const int64_t *row_ptr, const int32_t *col_idx, const double *old_vector,
                        double *new_vector, size_t n, size_t col_size)
{
    return crs_spmv_host<double>(val, row_ptr, col_idx, old_vector, new_vector, n, col_size);
}

int pfg_crs_spmv_real32(const float *val, const int64_t *row_ptr, const int32_t *col_idx, const float *old_vector,
                        float *new_vector, size_t n, size_t col_size)
{
    return crs_spmv_host<float>(val, row_ptr, col_idx, old_vector, new_vector, n, col_size);
}

int pfg_linear_solver_crs(const int64_t *row_ptr, const int32_t *col_idx, const double *val, const double *rhs,
                          double *x, int64_t n, int64_t nnz, const pfg_solve_opts *opts, pfg_info *info)
{
    // One cached context per thread: device buffers and captured graphs are
    // reused when the same-size system is solved again.
    static thread_local pfg_solver *ctx = nullptr;
    SolveResult res;
    const int rc = guard([&] {
        need(row_ptr && col_idx && val && rhs && x && n > 0, PFG_E_ARG, "NULL argument");
        need(row_ptr[0] == 1 && row_ptr[n] - 1 == nnz, PFG_E_ARG, "row_ptr inconsistent with nnz");
        if (!ctx) {
            pfg_solver *h = nullptr;
            if (pfg_create(&h) != PFG_OK) throw Error(PFG_E_CUDA, pfg_last_error());
            ctx = h;
        }
        pfg_solver *h = ctx;
        std::lock_guard<std::mutex> lk(h->mu);
        const KConfig cfg = to_config(opts);
        // debug: host time of each phase (the stream is drained at each mark)
        const auto t0 = std::chrono::steady_clock::now();
        auto mark = [&](const char *what) {
            if (cfg.debug == 0) return;
            PFG_CUDA(cudaStreamSynchronize(h->st));
            const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
            fprintf(stderr, "[pfg] linear_solver_crs %-8s %9.3f ms\n", what, ms);
        };
        static thread_local DevBuf<int64_t> rp;
        static thread_local DevBuf<int32_t> ci;
        static thread_local DevBuf<double> v, b;
        rp.ensure((size_t)n + 1);
        ci.ensure((size_t)std::max<int64_t>(nnz, 1));
        v.ensure((size_t)std::max<int64_t>(nnz, 1));
        b.ensure((size_t)n);
        PFG_CUDA(cudaMemcpyAsync(rp.p, row_ptr, (n + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, h->st));
        PFG_CUDA(cudaMemcpyAsync(ci.p, col_idx, nnz * sizeof(int32_t), cudaMemcpyHostToDevice, h->st));
        PFG_CUDA(cudaMemcpyAsync(v.p, val, nnz * sizeof(double), cudaMemcpyHostToDevice, h->st));
        PFG_CUDA(cudaMemcpyAsync(b.p, rhs, n * sizeof(double), cudaMemcpyHostToDevice, h->st));
        mark("copy-in");
        // same sizes as the previous call: the import reuses the device
        // buffers (same addresses), so the cached solver graphs stay valid
        import_crs(n, nnz, rp.p, ci.p, v.p, h->K, h->st);
        h->have_crs = true;
        h->x.ensure((size_t)n);
        PFG_CUDA(cudaMemcpyAsync(h->x.p, x, n * sizeof(double), cudaMemcpyHostToDevice, h->st));
        mark("import");
        res = h->kry.solve(h->K, b.p, h->x.p, cfg, h->st);
        mark("solve");
        PFG_CUDA(cudaMemcpyAsync(x, h->x.p, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
        PFG_CUDA(cudaStreamSynchronize(h->st));
        mark("copy-out");
        fill_info(info, res, cfg.precision);
    });
    if (rc != PFG_OK) return rc;
    return solve_status(res);
}

}  // extern "C"

extern "C" int pfg_profile_kernel(pfg_solver *h, int32_t kernel, int32_t reps, double *ms_per_launch,
                                  double *bytes_per_launch)
{
    return guard([&] {
        need(h && ms_per_launch && bytes_per_launch, PFG_E_ARG, "NULL argument");
        std::lock_guard<std::mutex> lk(h->mu);
        need(h->have_crs, PFG_E_STATE, "no CRS matrix");
        flush_pending(h);
        h->kry.profile(h->K, kernel, reps, h->st, *ms_per_launch, *bytes_per_launch);
    });
}

// ------------------------------------------------------------- eigenproblem
#include "lobpcg.cuh"

namespace {

void copy_matrix(const DevMatrix &src, DevMatrix &dst, cudaStream_t st)
{
    dst.bs = src.bs;
    dst.nb = src.nb;
    dst.nnzb = src.nnzb;
    dst.rp.resize(src.rp.n);
    dst.col.resize(src.col.n);
    dst.v64.resize(src.v64.n);
    PFG_CUDA(cudaMemcpyAsync(dst.rp.p, src.rp.p, src.rp.bytes(), cudaMemcpyDeviceToDevice, st));
    PFG_CUDA(cudaMemcpyAsync(dst.col.p, src.col.p, src.col.bytes(), cudaMemcpyDeviceToDevice, st));
    PFG_CUDA(cudaMemcpyAsync(dst.v64.p, src.v64.p, src.v64.bytes(), cudaMemcpyDeviceToDevice, st));
    dst.pattern_changed();
}

DevMatrix *find_slot(pfg_solver *h, const std::string &name)
{
    for (auto &kv : h->stack)
        if (kv.first == name) return &kv.second;
    return nullptr;
}

}  // namespace

extern "C" {

void pfg_eig_opts_default(pfg_eig_opts *o)
{
    if (!o) return;
    memset(o, 0, sizeof(*o));
    o->block_size = 0;
    o->max_itr = 100000;
    o->tol = 1.0e-6;
    o->precision = PFG_PREC_FP64;
    o->precond = PFG_PC_BLOCK_JACOBI;
    o->stop_rule = PFG_EIG_STOP_RESIDUAL;
    o->seed = 1;
    o->tol_fp32 = 1.0e-4;
}

int pfg_keep_this_matrix_as(pfg_solver *h, const char *name)
{
    return guard([&] {
        need(h && name, PFG_E_ARG, "NULL argument");
        std::lock_guard<std::mutex> lk(h->mu);
        need(h->have_crs, PFG_E_STATE, "keepThisMatrixAs before setCRS");
        flush_pending(h);
        DevMatrix *slot = find_slot(h, name);
        if (!slot) {
            need(h->stack.size() < 10, PFG_E_ARG, "keepThisMatrixAs: more than 10 named matrices");
            h->stack.emplace_back(std::string(name), DevMatrix());
            slot = &h->stack.back().second;
        }
        copy_matrix(h->K, *slot, h->st);
        PFG_CUDA(cudaStreamSynchronize(h->st));
    });
}

int pfg_load_matrix(pfg_solver *h, const char *name)
{
    return guard([&] {
        need(h && name, PFG_E_ARG, "NULL argument");
        std::lock_guard<std::mutex> lk(h->mu);
        flush_pending(h);
        DevMatrix *slot = find_slot(h, name);
        need(slot != nullptr, PFG_E_ARG, "loadMatrix: no matrix kept under that name");
        copy_matrix(*slot, h->K, h->st);
        h->have_crs = true;
        PFG_CUDA(cudaStreamSynchronize(h->st));
    });
}

int pfg_fix_eig(pfg_solver *h, int64_t n, const int32_t *ids)
{
    return guard([&] {
        need(h && (ids || n == 0), PFG_E_ARG, "NULL argument");
        std::lock_guard<std::mutex> lk(h->mu);
        for (int64_t i = 0; i < n; ++i) h->fix_eig_ids.push_back(ids[i]);
        std::sort(h->fix_eig_ids.begin(), h->fix_eig_ids.end());
        h->fix_eig_ids.erase(std::unique(h->fix_eig_ids.begin(), h->fix_eig_ids.end()), h->fix_eig_ids.end());
    });
}

int pfg_eig_reduced_size(pfg_solver *h, int64_t *n)
{
    return guard([&] {
        need(h && n, PFG_E_ARG, "NULL argument");
        std::lock_guard<std::mutex> lk(h->mu);
        DevMatrix *A = find_slot(h, "A");
        need(A, PFG_E_STATE, "no matrix kept as \"A\" (keepThisMatrixAs)");
        int64_t nf = 0;
        for (int id : h->fix_eig_ids) nf += (id >= 1 && id <= A->ndof());
        *n = A->ndof() - nf;
    });
}

int pfg_eig_dense(pfg_solver *h, int32_t num_eigen, double *eigen_value, double *eigen_vectors, pfg_info *info)
{
    int status = PFG_OK;
    const int rc = guard([&] {
        need(h && eigen_value, PFG_E_ARG, "NULL argument");
        std::lock_guard<std::mutex> lk(h->mu);
        DevMatrix *A = find_slot(h, "A"), *B = find_slot(h, "B");
        need(A && B, PFG_E_STATE, "eig needs matrices kept as \"A\" and \"B\" (keepThisMatrixAs)");
        need(A->nb == B->nb && A->bs == B->bs, PFG_E_ARG, "A and B differ in size or block structure");
        const auto t0 = std::chrono::steady_clock::now();
        const int64_t n = A->ndof();
        // reduce_crs_matrix order: the remaining DOFs keep their order
        std::vector<int> map((size_t)n, 0);
        for (int id : h->fix_eig_ids)
            if (id >= 1 && id <= n) map[(size_t)id - 1] = -1;
        std::vector<int64_t> old_of_new;
        for (int64_t i = 0; i < n; ++i)
            if (map[(size_t)i] == 0) {
                map[(size_t)i] = (int)old_of_new.size();
                old_of_new.push_back(i);
            }
        const int64_t N = (int64_t)old_of_new.size();
        need(N >= 1, PFG_E_ARG, "every DOF is fixed (fix_eig)");
        PFG_CHECK(N <= kDenseEigMax, PFG_E_UNSUPPORTED,
                  "dense eig (use_LOBPCG = .false.): " + std::to_string(N) + " unknowns, at most " +
                      std::to_string(kDenseEigMax) + " on this path; set use_LOBPCG for larger problems");
        const int64_t num = num_eigen > 0 ? std::min<int64_t>(num_eigen, N) : N;
        DevBuf<int> dmap((size_t)n);
        PFG_CUDA(cudaMemcpyAsync(dmap.p, map.data(), (size_t)n * sizeof(int), cudaMemcpyHostToDevice, h->st));
        DevBuf<double> dA((size_t)(N * N)), dB((size_t)(N * N)), dZ((size_t)(N * N));
        PFG_CUDA(cudaMemsetAsync(dA.p, 0, dA.bytes(), h->st));
        PFG_CUDA(cudaMemsetAsync(dB.p, 0, dB.bytes(), h->st));
        k_dense_from_blocks<<<grid_for(A->nb, 128), 128, 0, h->st>>>(A->nb, A->bs, A->rp.p, A->col.p, A->v64.p,
                                                                    dmap.p, (int)N, dA.p);
        k_dense_from_blocks<<<grid_for(B->nb, 128), 128, 0, h->st>>>(B->nb, B->bs, B->rp.p, B->col.p, B->v64.p,
                                                                    dmap.p, (int)N, dB.p);
        PFG_CUDA(cudaGetLastError());
        std::vector<double> w((size_t)N);
        int sweeps = 0;
        dense_generalized_eig((int)N, dA.p, dB.p, w.data(), dZ.p, &sweeps, h->st);
        std::vector<int> order((size_t)N);
        std::iota(order.begin(), order.end(), 0);
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return w[(size_t)a] < w[(size_t)b]; });
        for (int64_t k = 0; k < num; ++k) eigen_value[k] = w[(size_t)order[(size_t)k]];
        if (eigen_vectors) {
            // scatter back to every DOF, zero at the fixed ones (eigFEMSolver :1498-1539)
            std::vector<double> Z((size_t)(N * N));
            PFG_CUDA(cudaMemcpyAsync(Z.data(), dZ.p, dZ.bytes(), cudaMemcpyDeviceToHost, h->st));
            PFG_CUDA(cudaStreamSynchronize(h->st));
            std::fill(eigen_vectors, eigen_vectors + n * num, 0.0);
            for (int64_t k = 0; k < num; ++k) {
                const int c = order[(size_t)k];
                double *x = eigen_vectors + k * n;
                for (int64_t r = 0; r < N; ++r) x[old_of_new[(size_t)r]] = Z[(size_t)(r * N + c)];
            }
        }
        const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        if (info) {
            info->status = status;
            info->iterations = sweeps;
            info->replacements = 0;
            info->kernel_launches = 0;
            info->rel_residual = 0.0;
            info->iter_residual = 0.0;
            info->solve_ms = ms;
            info->fallback = 0;
        }
    });
    return rc != PFG_OK ? rc : status;
}

int pfg_eig(pfg_solver *h, const pfg_eig_opts *opts, int32_t num_eigen, double *eigen_value, double *eigen_vectors,
            pfg_info *info)
{
    EigResult r;
    const int rc = guard([&] {
        need(h && eigen_value && num_eigen >= 1, PFG_E_ARG, "bad eig arguments");
        std::lock_guard<std::mutex> lk(h->mu);
        DevMatrix *A = find_slot(h, "A"), *B = find_slot(h, "B");
        need(A && B, PFG_E_STATE, "eig needs matrices kept as \"A\" and \"B\" (keepThisMatrixAs)");
        need(A->nb == B->nb && A->bs == B->bs, PFG_E_ARG, "A and B differ in size or block structure");
        pfg_eig_opts d;
        pfg_eig_opts_default(&d);
        if (!opts) opts = &d;
        EigConfig cfg;
        cfg.nev = num_eigen;
        cfg.block = opts->block_size > 0 ? opts->block_size : num_eigen;
        cfg.max_itr = opts->max_itr > 0 ? opts->max_itr : 100000;
        cfg.tol = opts->tol > 0 ? opts->tol : 1e-6;
        cfg.precision = opts->precision;
        cfg.precond = opts->precond;
        cfg.stop_rule = opts->stop_rule;
        cfg.seed = opts->seed;
        cfg.tol_fp32 = opts->tol_fp32 > 0 ? opts->tol_fp32 : 1e-4;
        cfg.debug = opts->debug;
        const int64_t n = A->ndof();
        std::vector<uint8_t> mask((size_t)n, 0);
        for (int id : h->fix_eig_ids)
            if (id >= 1 && id <= n) mask[(size_t)id - 1] = 1;
        DevBuf<uint8_t> dmask((size_t)n);
        PFG_CUDA(cudaMemcpyAsync(dmask.p, mask.data(), n, cudaMemcpyHostToDevice, h->st));
        DevBuf<double> X(eigen_vectors ? (size_t)n * num_eigen : 0);
        r = lobpcg_solve(*A, *B, dmask.p, cfg, eigen_value, eigen_vectors ? X.p : nullptr, h->st);
        if (eigen_vectors)
            PFG_CUDA(cudaMemcpyAsync(eigen_vectors, X.p, (size_t)n * num_eigen * sizeof(double), cudaMemcpyDeviceToHost,
                                     h->st));
        PFG_CUDA(cudaStreamSynchronize(h->st));
        if (info) {
            info->status = r.status;
            info->iterations = r.iterations;
            info->replacements = r.iterations_fp32;
            info->kernel_launches = r.launches;
            info->rel_residual = r.max_rel_residual;
            info->iter_residual = r.max_rel_residual;
            info->solve_ms = r.ms;
            info->fallback = 0;
        }
    });
    if (rc != PFG_OK) return rc;
    if (r.status == PFG_W_NOT_CONVERGED) set_last_error("[ERROR] LOBPCG NOT CONVERGED (LOBPCG_MAX_ITR reached)");
    return r.status;
}

}  // extern "C"

// ------------------------------------------------- elimination, stress, adjoint
namespace {

cudaStream_t pick_stream(pfg_solver *h, void *stream)
{
    if (stream) {
        PFG_CUDA(cudaStreamSynchronize(h->st));
        return (cudaStream_t)stream;
    }
    PFG_CUDA(cudaStreamSynchronize((cudaStream_t)0));  // order after the caller's default-stream work
    return h->st;
}

void check_prop_device(pfg_solver *h, int64_t n_prop)
{
    need(n_prop == 1 || n_prop == h->mesh.ne, PFG_E_ARG, "property arrays need 1 or number_of_element values");
}

}  // namespace

extern "C" {

int pfg_eliminate(pfg_solver *h)
{
    return guard([&] {
        need(h != nullptr, PFG_E_ARG, "NULL handle");
        std::lock_guard<std::mutex> lk(h->mu);
        need(h->have_crs, PFG_E_STATE, "eliminate before setCRS");
        flush_pending(h);
        apply_fix_device(h);
        PFG_CUDA(cudaStreamSynchronize(h->st));
    });
}

int pfg_ilu_reset(pfg_solver *h)
{
    return guard([&] {
        need(h != nullptr, PFG_E_ARG, "NULL handle");
        std::lock_guard<std::mutex> lk(h->mu);
        h->kry.ilu_reset();
    });
}

int pfg_ilu_factor(pfg_solver *h, int32_t sorted, double *lu_out)
{
    return guard([&] {
        need(h != nullptr, PFG_E_ARG, "NULL handle");
        std::lock_guard<std::mutex> lk(h->mu);
        need(h->have_crs, PFG_E_STATE, "ILU(0) before setCRS");
        flush_pending(h);
        const Ilu0 &f = h->kry.ilu_factor(h->K, sorted != 0, h->st);
        if (lu_out) {
            const int64_t nnz = h->K.nnzb * h->K.bs * h->K.bs;
            DevBuf<double> v((size_t)std::max<int64_t>(nnz, 1));
            export_values(h->K, f.lu(), v.p, h->st);
            PFG_CUDA(cudaMemcpyAsync(lu_out, v.p, nnz * sizeof(double), cudaMemcpyDeviceToHost, h->st));
        }
        PFG_CUDA(cudaStreamSynchronize(h->st));
    });
}

int pfg_ilu_apply(pfg_solver *h, const double *v, double *out)
{
    return guard([&] {
        need(h && v && out, PFG_E_ARG, "NULL argument");
        std::lock_guard<std::mutex> lk(h->mu);
        need(h->have_crs, PFG_E_STATE, "ILU(0) before setCRS");
        const int64_t n = h->ndof();
        DevBuf<double> dv((size_t)n), dout((size_t)n);
        PFG_CUDA(cudaMemcpyAsync(dv.p, v, n * sizeof(double), cudaMemcpyHostToDevice, h->st));
        const Ilu0 *held = h->kry.ilu_held();
        const Ilu0 &f = held ? *held : h->kry.ilu_factor(h->K, true, h->st);
        f.apply(dv.p, dout.p, nullptr, h->st);
        PFG_CUDA(cudaMemcpyAsync(out, dout.p, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
        PFG_CUDA(cudaStreamSynchronize(h->st));
    });
}

int pfg_ilu_solve(pfg_solver *h, const double *rhs, double *x)
{
    return guard([&] {
        need(h && rhs && x, PFG_E_ARG, "NULL argument");
        std::lock_guard<std::mutex> lk(h->mu);
        need(h->have_crs, PFG_E_STATE, "ILU(0) before setCRS");
        flush_pending(h);
        const int64_t n = h->ndof();
        DevBuf<double> dr((size_t)n), dx((size_t)n);
        PFG_CUDA(cudaMemcpyAsync(dr.p, rhs, n * sizeof(double), cudaMemcpyHostToDevice, h->st));
        const Ilu0 *held = h->kry.ilu_held();
        const Ilu0 &f = held ? *held : h->kry.ilu_factor(h->K, true, h->st);
        f.solve(dr.p, dx.p, h->st);
        PFG_CUDA(cudaMemcpyAsync(x, dx.p, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
        PFG_CUDA(cudaStreamSynchronize(h->st));
    });
}

int pfg_element_stress(pfg_solver *h, const double *displacement, int64_t n_prop, const double *E, const double *v,
                       int32_t option, double *out)
{
    return guard([&] {
        need(h && displacement && E && v && out, PFG_E_ARG, "NULL argument");
        need((option >= 0 && option <= 7) || (option >= 10 && option <= 18), PFG_E_ARG,
             "option: 0 tensor, 1 I1, 2 p, 3 I2, 4 I3, 5 J1, 6 J2, 7 J3, 10 + 3 (i-1) + (j-1) component (i, j)");
        std::lock_guard<std::mutex> lk(h->mu);
        need(h->have_mesh, PFG_E_STATE, "stress before setDomain");
        const int64_t ne = h->mesh.ne, n = 3 * h->mesh.nn;
        DevBuf<double> du((size_t)n), dE, dnu, S((size_t)ne * 9);
        upload_prop(h, n_prop, E, dE, "E");
        upload_prop(h, n_prop, v, dnu, "v");
        PFG_CUDA(cudaMemcpyAsync(du.p, displacement, n * sizeof(double), cudaMemcpyHostToDevice, h->st));
        element_stress(h->mesh, du.p, dE.p, dnu.p, n_prop == 1, S.p, h->st);
        if (option == 0) {
            PFG_CUDA(cudaMemcpyAsync(out, S.p, ne * 9 * sizeof(double), cudaMemcpyDeviceToHost, h->st));
        } else {
            DevBuf<double> r((size_t)ne);
            element_stress_option(ne, S.p, option, r.p, h->st);
            PFG_CUDA(cudaMemcpyAsync(out, r.p, ne * sizeof(double), cudaMemcpyDeviceToHost, h->st));
        }
        PFG_CUDA(cudaStreamSynchronize(h->st));
    });
}

int pfg_dev_assemble_stiffness(pfg_solver *h, int64_t n_prop, const double *d_E, const double *d_nu, void *stream)
{
    return guard([&] {
        need(h && d_E && d_nu, PFG_E_ARG, "NULL argument");
        std::lock_guard<std::mutex> lk(h->mu);
        need(h->have_mesh, PFG_E_STATE, "assemble before setDomain");
        ensure_crs(h);
        flush_pending(h);
        check_prop_device(h, n_prop);
        cudaStream_t st = pick_stream(h, stream);
        assemble_elements(h->mesh, h->K, 0, d_E, d_nu, n_prop == 1, st);
    });
}

int pfg_dev_set_rhs(pfg_solver *h, int64_t n, const double *d_rhs, void *stream)
{
    return guard([&] {
        need(h && d_rhs, PFG_E_ARG, "NULL argument");
        std::lock_guard<std::mutex> lk(h->mu);
        ensure_crs(h);
        need(n == h->ndof(), PFG_E_ARG, "setRHS: size differs from the CRS matrix");
        cudaStream_t st = pick_stream(h, stream);
        PFG_CUDA(cudaMemcpyAsync(h->rhs.p, d_rhs, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
        PFG_CUDA(cudaStreamSynchronize(st));
    });
}

int pfg_dev_adjoint_grad_E(pfg_solver *h, const double *d_u, const double *d_lambda, int64_t n_prop,
                           const double *d_nu, double *d_grad, void *stream)
{
    return guard([&] {
        need(h && d_u && d_lambda && d_nu && d_grad, PFG_E_ARG, "NULL argument");
        std::lock_guard<std::mutex> lk(h->mu);
        need(h->have_mesh, PFG_E_STATE, "adjoint before setDomain");
        check_prop_device(h, n_prop);
        cudaStream_t st = pick_stream(h, stream);
        adjoint_grad_E(h->mesh, d_u, d_lambda, d_nu, n_prop == 1, d_grad, st);
    });
}

}  // extern "C"

// ----------------------------------------------------------- batched solves
namespace pfg {

// Prepares handle h for a batched solve: flushes buffered element matrices,
// applies the Dirichlet elimination FEMSolver_%solve applies before solving
// (FEMSolverClass.f90:1707-1756), refreshes the sliced FP64 and FP32 copies
// and describes what the batched kernel reads.
BatchSource batch_bind(pfg_solver *h)
{
    PFG_CHECK(h != nullptr, PFG_E_ARG, "NULL handle in a batch");
    std::lock_guard<std::mutex> lk(h->mu);
    PFG_CHECK(h->have_crs, PFG_E_STATE, "batch member without a CRS matrix");
    PFG_CHECK(h->K.bs == 3, PFG_E_UNSUPPORTED, "batched solves take 3-DOF (3x3-block) systems");
    flush_pending(h);
    apply_fix_device(h);
    build_sell(h->K, true, true, h->st);
    PFG_CUDA(cudaStreamSynchronize(h->st));
    BatchSource s;
    s.K = &h->K;
    s.b = h->rhs.p;
    s.fixed = h->have_fix ? h->fixed_d.p : nullptr;
    s.fixval = h->have_fix ? h->fixval_d.p : nullptr;
    s.device = h->device;
    return s;
}

}  // namespace pfg

// ---------------------------------------------------- Newmark-beta time stepping
namespace {

// out = cM * M + cK * K over the value arrays of two matrices of one pattern
__global__ void k_combine_values(int64_t len, double cM, const double *__restrict__ M, double cK,
                                 const double *__restrict__ K, double *__restrict__ out)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = fma(cM, M[i], cK * K[i]);
}

// weights of the Newmark right-hand side R = M wM + K wK (the C = alpha M + beta K
// terms folded into both; a_ext: external acceleration, F = M a_ext)
__global__ void k_newmark_weights(int64_t n, const double *__restrict__ a_ext, const double *__restrict__ u,
                                  const double *__restrict__ v, const double *__restrict__ a, double mu, double mv,
                                  double ma, double ku, double kv, double ka, double *__restrict__ wM,
                                  double *__restrict__ wK)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double ae = a_ext ? a_ext[i] : 0.0;
        wM[i] = ae + mu * u[i] + mv * v[i] + ma * a[i];
        wK[i] = ku * u[i] + kv * v[i] + ka * a[i];
    }
}

// rhs = R + base on free rows (base = -A_eff[:, fixed] u_fixed), prescribed value on fixed rows
__global__ void k_newmark_rhs(int64_t n, double *__restrict__ rhs, const double *__restrict__ tmp,
                              const double *__restrict__ base, const uint8_t *__restrict__ fixed)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        rhs[i] = (fixed && fixed[i]) ? base[i] : rhs[i] + tmp[i] + base[i];
}

// updateVelocity / updateAccelNewmarkBeta (SeismicAnalysisClass.f90:1501-1535), then u = u'
__global__ void k_newmark_update(int64_t n, const double *__restrict__ un, double *__restrict__ u,
                                 double *__restrict__ v, double *__restrict__ a, double beta, double gamma, double dt)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double du = un[i] - u[i];
        const double vn = gamma / (beta * dt) * du + (1.0 - gamma / beta) * v[i] + dt * (1.0 - gamma / (2.0 * beta)) * a[i];
        const double an = du / (beta * dt * dt) - v[i] / (beta * dt) + (1.0 - 1.0 / (2.0 * beta)) * a[i];
        u[i] = un[i];
        v[i] = vn;
        a[i] = an;
    }
}

}  // namespace

extern "C" {

void pfg_newmark_params_default(pfg_newmark_params *p)
{
    if (!p) return;
    // SeismicAnalysis_ defaults (SeismicAnalysisClass.f90:98-109)
    p->dt = 1.0;
    p->newmark_beta = 0.25;
    p->newmark_gamma = 0.5;
    p->rayleigh_alpha = 0.524;
    p->rayleigh_beta = 0.00129;
}

int pfg_newmark_setup(pfg_solver *h, const pfg_newmark_params *p)
{
    return guard([&] {
        need(h && p, PFG_E_ARG, "NULL argument");
        need(p->dt > 0.0 && p->newmark_beta > 0.0 && p->newmark_gamma > 0.0, PFG_E_ARG,
             "Newmark: dt, beta and gamma must be positive");
        std::lock_guard<std::mutex> lk(h->mu);
        flush_pending(h);
        DevMatrix *Kp = find_slot(h, "A"), *Mp = find_slot(h, "B");
        need(Kp && Mp, PFG_E_STATE, "Newmark: keep the stiffness as \"A\" and the mass as \"B\" first");
        need(Kp->bs == Mp->bs && Kp->nb == Mp->nb && Kp->nnzb == Mp->nnzb, PFG_E_ARG,
             "Newmark: stiffness and mass must share one CRS pattern");
        const double b = p->newmark_beta, g = p->newmark_gamma, dt = p->dt;
        // getNewmarkBetaMatrix (SeismicAnalysisClass.f90:1464-1476) with C = alpha M + beta K
        const double cM = 1.0 / (b * dt * dt) + g / (b * dt) * p->rayleigh_alpha;
        const double cK = 1.0 + g / (b * dt) * p->rayleigh_beta;
        copy_matrix(*Kp, h->K, h->st);
        const int64_t len = Kp->nnzb * Kp->bs * Kp->bs;
        k_combine_values<<<grid_for(len, 256, sm_count_device() * 16), 256, 0, h->st>>>(len, cM, Mp->v64.p, cK, Kp->v64.p,
                                                                          h->K.v64.p);
        PFG_CUDA(cudaGetLastError());
        h->K.values_changed();
        h->have_crs = true;
        const int64_t n = h->K.ndof();
        auto &nm = h->nm;
        for (DevBuf<double> *v : {&nm.u, &nm.v, &nm.a, &nm.base, &nm.wM, &nm.wK, &nm.rhs, &nm.tmp, &nm.x})
            v->resize((size_t)n);
        for (DevBuf<double> *v : {&nm.u, &nm.v, &nm.a, &nm.base})
            PFG_CUDA(cudaMemsetAsync(v->p, 0, n * sizeof(double), h->st));
        // symmetric elimination of the fixed DOFs (LinearSolver_%fix,
        // LinearSolverClass.f90:266-290); on a zero right-hand side it leaves
        // base = -A_eff[:, fixed] u_fixed on free rows and u_fixed on fixed rows
        if (h->have_fix) {
            h->fixed_d.ensure((size_t)n);
            h->fixval_d.ensure((size_t)n);
            PFG_CUDA(cudaMemcpyAsync(h->fixed_d.p, h->fixed_h.data(), n, cudaMemcpyHostToDevice, h->st));
            PFG_CUDA(cudaMemcpyAsync(h->fixval_d.p, h->fixval_h.data(), n * sizeof(double), cudaMemcpyHostToDevice,
                                     h->st));
            apply_dirichlet(h->K, nm.base.p, h->fixed_d.p, h->fixval_d.p, h->st);
            restore_fixed(n, nm.u.p, h->fixed_d.p, h->fixval_d.p, h->st);
        }
        PFG_CUDA(cudaStreamSynchronize(h->st));
        nm.dt = dt;
        nm.beta = b;
        nm.gamma = g;
        nm.ray_alpha = p->rayleigh_alpha;
        nm.ray_beta = p->rayleigh_beta;
        nm.ready = true;
    });
}

int pfg_newmark_set_state(pfg_solver *h, int64_t n, const double *u, const double *v, const double *a)
{
    return guard([&] {
        need(h != nullptr, PFG_E_ARG, "NULL handle");
        std::lock_guard<std::mutex> lk(h->mu);
        need(h->nm.ready, PFG_E_STATE, "Newmark: set-up first");
        need(n == h->K.ndof(), PFG_E_ARG, "Newmark: state size differs from the system");
        if (u) PFG_CUDA(cudaMemcpyAsync(h->nm.u.p, u, n * sizeof(double), cudaMemcpyHostToDevice, h->st));
        if (v) PFG_CUDA(cudaMemcpyAsync(h->nm.v.p, v, n * sizeof(double), cudaMemcpyHostToDevice, h->st));
        if (a) PFG_CUDA(cudaMemcpyAsync(h->nm.a.p, a, n * sizeof(double), cudaMemcpyHostToDevice, h->st));
        PFG_CUDA(cudaStreamSynchronize(h->st));
    });
}

int pfg_newmark_step(pfg_solver *h, const pfg_solve_opts *opts, int64_t n, const double *a_ext, double *u_out,
                     double *v_out, double *a_out, pfg_info *info)
{
    SolveResult res;
    const int rc = guard([&] {
        need(h != nullptr, PFG_E_ARG, "NULL handle");
        std::lock_guard<std::mutex> lk(h->mu);
        auto &nm = h->nm;
        need(nm.ready, PFG_E_STATE, "Newmark: set-up first");
        need(n == h->K.ndof(), PFG_E_ARG, "Newmark: vector size differs from the system");
        DevMatrix *Kp = find_slot(h, "A"), *Mp = find_slot(h, "B");
        need(Kp && Mp, PFG_E_STATE, "Newmark: the kept stiffness / mass are gone");
        const double b = nm.beta, g = nm.gamma, dt = nm.dt;
        // getNewmarkBetaVector (SeismicAnalysisClass.f90:1478-1499):
        //   R = M a_ext + M (u/(b dt^2) + v/(b dt) + (1/(2b) - 1) a)
        //     + C (g/(b dt) u + (g/b - 1) v + dt (g/(2b) - 1) a),   C = alpha M + beta K
        const double du = g / (b * dt), dv = g / b - 1.0, da = dt * (g / (2.0 * b) - 1.0);
        const double mu = 1.0 / (b * dt * dt) + nm.ray_alpha * du, mv = 1.0 / (b * dt) + nm.ray_alpha * dv,
                     ma = 1.0 / (2.0 * b) - 1.0 + nm.ray_alpha * da;
        const double ku = nm.ray_beta * du, kv = nm.ray_beta * dv, ka = nm.ray_beta * da;
        const int gv = grid_for(n, 256, sm_count_device() * 16);
        if (a_ext) PFG_CUDA(cudaMemcpyAsync(nm.tmp.p, a_ext, n * sizeof(double), cudaMemcpyHostToDevice, h->st));
        k_newmark_weights<<<gv, 256, 0, h->st>>>(n, a_ext ? nm.tmp.p : nullptr, nm.u.p, nm.v.p, nm.a.p, mu, mv, ma,
                                                 ku, kv, ka, nm.wM.p, nm.wK.p);
        PFG_CUDA(cudaGetLastError());
        Krylov::spmv64_sliced(*Mp, nm.wM.p, nm.rhs.p, h->st);
        Krylov::spmv64_sliced(*Kp, nm.wK.p, nm.tmp.p, h->st);
        k_newmark_rhs<<<gv, 256, 0, h->st>>>(n, nm.rhs.p, nm.tmp.p, nm.base.p, h->have_fix ? h->fixed_d.p : nullptr);
        PFG_CUDA(cudaGetLastError());
        // A_eff u' = rhs from the previous displacement
        PFG_CUDA(cudaMemcpyAsync(nm.x.p, nm.u.p, n * sizeof(double), cudaMemcpyDeviceToDevice, h->st));
        KConfig cfg = to_config(opts);
        if (!opts) {
            cfg.algorithm = PFG_ALG_CG;
            cfg.precond = PFG_PC_BLOCK_JACOBI;
            cfg.stop_rule = PFG_STOP_TRUE_RELATIVE;
            cfg.graph_chunk = 8;  // short warm-started solves
        }
        res = h->kry.solve(h->K, nm.rhs.p, nm.x.p, cfg, h->st);
        if (h->have_fix) restore_fixed(n, nm.x.p, h->fixed_d.p, h->fixval_d.p, h->st);
        k_newmark_update<<<gv, 256, 0, h->st>>>(n, nm.x.p, nm.u.p, nm.v.p, nm.a.p, b, g, dt);
        PFG_CUDA(cudaGetLastError());
        if (u_out) PFG_CUDA(cudaMemcpyAsync(u_out, nm.u.p, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
        if (v_out) PFG_CUDA(cudaMemcpyAsync(v_out, nm.v.p, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
        if (a_out) PFG_CUDA(cudaMemcpyAsync(a_out, nm.a.p, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
        PFG_CUDA(cudaStreamSynchronize(h->st));
        fill_info(info, res, cfg.precision);
    });
    if (rc != PFG_OK) return rc;
    return solve_status(res);
}

}  // extern "C"
