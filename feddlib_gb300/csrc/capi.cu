// capi.cu -- the C ABI (include/feddgpu.h): handle lifetime, pattern build,
// and the per-call orchestration of the element and row stages.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <unordered_map>

#include "kernels.cuh"

using namespace fedd;

struct fedd_assembler {
    int device = 0;
    fedd_params prm{};
    int order = 2, npe = 10;
    int64_t nn = 0, ne = 0, nn_p = 0;
    DBuf<double> xyz;
    DBuf<int32_t> conn, conn_p;
    Graph g, gp;
    DBuf<int32_t> vmap;     // Taylor-Hood: P2 vertex -> P1 node (-1 for edge nodes)
    DBuf<unsigned long long> work;  // the velocity-row kernel's position counter (device path)
    bool ns_fused = false;  // vmap verified: pressure rows come from the velocity-row kernel
    DBuf<int64_t> padj_ptr;
    DBuf<int4> ninfo;       // per velocity node: first incidence, vertex P1 node, counts (k_ns_vel_rows)
    DBuf<int32_t> padj;
    int max_padj = 0;
    int64_t n_padj = 0;
    Csr csr[4];
    DBuf<float> stage_f;
    DBuf<double> stage_d;
    DBuf<double> lap_tab;
    float *ns_tab = nullptr;
    HyperTables htab{};
    LawParams law{};
    // surrogate
    bool has_mlp = false;
    DBuf<__nv_bfloat16> mW1, mW2, mw3;
    DBuf<float> mb1, mb2;
    MLPDev mlp{};
    DBuf<float> qp_inv;
    DBuf<QPDerivs> qp_der;
    DBuf<uint8_t> qp_fb;
    DBuf<int> d_fb;
    int64_t last_fb = 0, last_nqp = 0;
    // host-buffer path scratch
    DBuf<double> u_dev, p_dev, v_dev[3], ru_dev, rp_dev;
    // host-buffer path pipeline: a copy stream and one event per chunk of row
    // nodes, so each chunk's values go to the host while the next is computed;
    // element chunk k (ends ecut) holds the elements node chunk k needs beyond
    // the earlier chunks, so the element stage is spread over the pipeline
    static constexpr int kChunks = 8;
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t chunk_ev[kChunks + 2] = {};
    bool chunks_ready = false;
    int64_t cut[kChunks + 1] = {}, off00[kChunks + 1] = {}, off01[kChunks + 1] = {}, ecut[kChunks + 1] = {};
    DBuf<int> d_err;
    // generalized-Newtonian viscosity law (fedd_set_viscosity_law)
    bool gn_on = false;
    ViscLaw gn{};
    DBuf<float> stage_gn;
    // elements flagged for the outflow Neumann term (fedd_set_outflow_faces)
    DBuf<int32_t> of_elem, of_face;
    int64_t of_n = 0;
    // linearization 2: the fixed-point matrix (prm.linearization holds 0 then)
    bool fp_matrix = false;
    // the residual's block factors (fedd_set_coeff)
    NSCoeff coeff;
    // per-element Young's modulus as E_e / E (fedd_set_element_moduli)
    DBuf<float> emod;
    GNOutflow outflow() const {
        GNOutflow o;
        o.elem = of_elem.p;
        o.face = of_face.p;
        o.n = of_n;
        o.matrix = fp_matrix ? 1 : 0;
        return o;
    }
    // Dirichlet dofs (fedd_dirichlet_set): rows of the velocity / scalar
    // block row and of the pressure block row
    DBuf<int64_t> dir_u, dir_p;
    int64_t n_dir_u = 0, n_dir_p = 0;
    int64_t launches = 0;
    std::string err;
    // profiling: event pairs per (call, stage)
    static constexpr int kProfCalls = 256, kProfStages = 8;
    bool prof = false;
    int prof_calls = 0, prof_stage = 0;
    std::vector<cudaEvent_t> ev;  // kProfCalls * kProfStages * 2
    std::vector<std::string> stage_names;
    ~fedd_assembler() {
        if (ns_tab) cudaFree(ns_tab);
        for (auto e : ev) cudaEventDestroy(e);
        for (auto e : chunk_ev)
            if (e) cudaEventDestroy(e);
        if (copy_stream) cudaStreamDestroy(copy_stream);
    }
};

std::string &fedd::thread_error() {
    static thread_local std::string msg;
    return msg;
}

namespace {

template <class F> fedd_status guarded(fedd_assembler *h, F &&f) {
    try {
        f();
        if (h) h->err.clear();
        return FEDD_OK;
    } catch (const Status &s) {
        if (h) h->err = s.msg;
        return s.code;
    } catch (const CudaError &e) {
        if (h) h->err = std::string(e.what) + ": " + cudaGetErrorString(e.code);
        return FEDD_ERR_CUDA;
    } catch (const std::bad_alloc &) {
        if (h) h->err = "host allocation failed";
        return FEDD_ERR_NOMEM;
    } catch (...) {
        if (h) h->err = "unexpected exception";
        return FEDD_ERR_CUDA;
    }
}

std::vector<int32_t> to_soa(const int32_t *aos, int64_t ne, int npe) {
    std::vector<int32_t> s((size_t)ne * npe);
    for (int64_t e = 0; e < ne; e++)
        for (int a = 0; a < npe; a++) s[(size_t)a * ne + e] = aos[(size_t)e * npe + a];
    return s;
}

int quad_points(const fedd_assembler *h) {
    if (h->prm.quad_points) return h->prm.quad_points;
    switch (h->prm.problem) {
    case FEDD_LINEAR_ELASTICITY: return 4;    // skr1, AceGen code 18
    case FEDD_NONLINEAR_ELASTICITY: return 5; // skr2, AceGen code 19
    case FEDD_NONLINEAR_ELASTICITY2: return 5; // skr3, AceGen code 19
    case FEDD_ANISO_FIBER: return 4;
    default: return 0;
    }
}

void set_law(fedd_assembler *h) {
    const fedd_params &p = h->prm;
    double E = p.E, nu = p.poisson_ratio;
    double mu = E / (2.0 * (1.0 + nu));            // NeoHookQuadraticTets.f:27-32
    double lam = nu * 2.0 * mu / (1.0 - 2.0 * nu);
    LawParams L{};
    L.kind = p.problem == FEDD_NONLINEAR_ELASTICITY    ? kLawSKR2
             : p.problem == FEDD_NONLINEAR_ELASTICITY2 ? kLawSKR3
             : p.problem == FEDD_ANISO_FIBER           ? (p.surrogate ? kLawMLP : kLawAniso)
                                                        : kLawSKR1;
    L.mu = (float)mu;
    // skr3 takes the bulk modulus (NeoHookQuadraticTets3.f: 1 / (6 (1 - 2 nu)) times 2 E)
    L.lam = (float)(L.kind == kLawSKR3 ? E / (3.0 * (1.0 - 2.0 * nu)) : lam);
    L.k1 = (float)p.k1;
    L.k2 = (float)p.k2;
    double a = p.fiber_angle_deg * M_PI / 180.0;
    L.a1[0] = (float)std::cos(a); L.a1[1] = (float)std::sin(a); L.a1[2] = 0.0f;
    L.a2[0] = (float)std::cos(a); L.a2[1] = (float)-std::sin(a); L.a2[2] = 0.0f;
    L.escale = h->emod.n ? h->emod.p : nullptr;
    h->law = L;
}

void read_dev_error(fedd_assembler *h, cudaStream_t s) {
    int e = 0;
    FEDD_CUDA(cudaMemcpyAsync(&e, h->d_err.p, sizeof e, cudaMemcpyDeviceToHost, s));
    FEDD_CUDA(cudaStreamSynchronize(s));
    if (e == kDevBadDet) FEDD_FAIL(FEDD_ERR_NONFINITE, "det B or det F is zero, negative or not finite");
    if (e == kDevNonFinite) FEDD_FAIL(FEDD_ERR_NONFINITE, "non-finite value in the element stage");
    if (e == kDevMesh) FEDD_FAIL(FEDD_ERR_MESH, "invalid mesh");
    if (e == kDevTimeout) FEDD_FAIL(FEDD_ERR_CUDA, "a tensor-core wait timed out");
    if (e) FEDD_FAIL(FEDD_ERR_CUDA, "device error word " + std::to_string(e));
}

// wraps one kernel launch with profiling events when profiling is on
template <class Fn> void stage(fedd_assembler *h, const char *name, cudaStream_t s, Fn &&fn) {
    const bool on = h->prof && h->prof_calls < fedd_assembler::kProfCalls &&
                    h->prof_stage < fedd_assembler::kProfStages;
    cudaEvent_t *e = nullptr;
    if (on) {
        e = &h->ev[((size_t)h->prof_calls * fedd_assembler::kProfStages + h->prof_stage) * 2];
        FEDD_CUDA(cudaEventRecord(e[0], s));
    }
    fn();
    if (on) {
        FEDD_CUDA(cudaEventRecord(e[1], s));
        if ((int)h->stage_names.size() <= h->prof_stage) h->stage_names.resize(h->prof_stage + 1);
        h->stage_names[h->prof_stage] = name;
        h->prof_stage++;
    }
}

void run(fedd_assembler *h, unsigned what, const double *d_u, const double *d_p, double *v00, double *v01,
         double *v10, double *ru, double *rp, cudaStream_t s) {
    LaunchCounter lc;
    const bool jac = what & FEDD_JACOBIAN, res = what & FEDD_RESIDUAL;
    FEDD_CUDA(cudaMemsetAsync(h->d_err.p, 0, sizeof(int), s));
    switch (h->prm.problem) {
    case FEDD_LAPLACE:
        stage(h, "lap_elem", s, [&] {
            launch_lap_elem(h->xyz.p, h->conn.p, h->ne, h->order, h->lap_tab.p, h->prm.source, h->stage_d.p,
                            h->d_err.p, s, lc);
        });
        stage(h, "lap_rows", s, [&] {
            launch_lap_rows(h->g, h->stage_d.p, h->order, h->csr[0].rowptr.p, jac ? v00 : nullptr,
                            res ? ru : nullptr, h->nn, s, lc);
        });
        break;
    case FEDD_LINEAR_ELASTICITY:
    case FEDD_NONLINEAR_ELASTICITY:
    case FEDD_NONLINEAR_ELASTICITY2:
    case FEDD_ANISO_FIBER: {
        const QPDerivs *qpd = nullptr;
        const uint8_t *qfb = nullptr;
        if (h->law.kind == kLawMLP) {
            if (!h->has_mlp) FEDD_FAIL(FEDD_ERR_STATE, "surrogate requested but no network set (fedd_set_surrogate)");
            const int64_t nqp = h->ne * h->htab.nq;
            stage(h, "qp_invariants", s, [&] {
                launch_hyper_invariants(h->xyz.p, h->conn.p, h->ne, d_u, h->law, h->htab, h->qp_inv.p, h->d_err.p,
                                        s, lc);
            });
            FEDD_CUDA(cudaMemsetAsync(h->d_fb.p, 0, sizeof(int), s));
            stage(h, "mlp_qp", s, [&] {
                launch_mlp_qp(h->mlp, h->law, h->qp_inv.p, nqp, h->qp_der.p, h->qp_fb.p, h->d_fb.p, h->d_err.p, s, lc);
            });
            qpd = h->qp_der.p;
            qfb = h->qp_fb.p;
            h->last_nqp = nqp;
        }
        stage(h, "hyper_elem", s, [&] {
            launch_hyper_elem(h->xyz.p, h->conn.p, h->ne, d_u, h->law, h->htab, qpd, qfb, h->stage_f.p,
                              res && d_u != nullptr, h->d_err.p, s, lc);
        });
        stage(h, "hyper_rows", s, [&] {
            launch_hyper_rows(h->g, h->stage_f.p, h->csr[0].rowptr.p, jac ? v00 : nullptr, res ? ru : nullptr, h->nn,
                              s, lc);
        });
        break;
    }
    case FEDD_NAVIER_STOKES: {
        // a generalized-Newtonian fluid replaces the Newtonian Laplacian by its
        // stress term: its element stage runs first and the velocity rows fold
        // its rows into their accumulation
        const float vd = h->gn_on ? 0.0f : (float)(h->prm.viscosity * h->prm.density);
        const float dn = (float)h->prm.density;
        stage(h, "ns_record", s, [&] {
            launch_ns_record(h->xyz.p, h->conn.p, h->conn_p.p, h->ne, d_u, d_p, h->ns_tab, vd, dn, h->stage_f.p,
                             h->d_err.p, s, lc);
        });
        if (h->gn_on)
            stage(h, "gn_elem", s, [&] {
                launch_gn_elem(h->xyz.p, h->conn.p, h->ne, d_u, h->gn, h->prm.linearization, h->stage_gn.p,
                               h->d_err.p, s, lc, 0, -1, h->outflow());
            });
        // with a verified vertex map the velocity-row warps of the vertices
        // assemble the pressure rows as well
        stage(h, "ns_vel_rows", s, [&] {
            launch_ns_vel_rows(h->g, h->ninfo.p, h->stage_f.p, h->ns_tab, h->csr[0].rowptr.p, h->csr[1].rowptr.p,
                               v00, v01, res ? ru : nullptr, vd, dn, h->prm.linearization, jac, h->g.max_adj,
                               h->max_padj, h->ns_fused ? h->vmap.p : nullptr, h->csr[2].rowptr.p, v10,
                               res ? rp : nullptr, h->gn_on ? h->stage_gn.p : nullptr, s, lc, 0, -1, h->work.p,
                               h->coeff);
        });
        if (!h->ns_fused)
            stage(h, "ns_pres_rows", s, [&] {
                launch_ns_pres_rows(h->gp, h->stage_f.p, h->ns_tab, h->csr[2].rowptr.p, v10, res ? rp : nullptr, jac,
                                    h->gp.max_adj, s, lc, h->coeff);
            });
        break;
    }
    default:
        FEDD_FAIL(FEDD_ERR_UNSUPPORTED, "unknown problem");
    }
    h->launches = lc.n;
    if (h->prof && h->prof_stage > 0 && h->prof_calls < fedd_assembler::kProfCalls) h->prof_calls++;
    h->prof_stage = 0;
}

}  // namespace

extern "C" {

int fedd_abi_version(void) { return FEDDGPU_ABI_VERSION; }

const char *fedd_status_string(fedd_status s) {
    switch (s) {
    case FEDD_OK: return "ok";
    case FEDD_ERR_ARG: return "invalid argument";
    case FEDD_ERR_CUDA: return "CUDA error";
    case FEDD_ERR_MESH: return "invalid mesh";
    case FEDD_ERR_NONFINITE: return "non-finite value";
    case FEDD_ERR_TIMEOUT: return "device wait timed out";
    case FEDD_ERR_NOMEM: return "out of memory";
    case FEDD_ERR_STATE: return "invalid state";
    case FEDD_ERR_UNSUPPORTED: return "unsupported";
    case FEDD_ERR_CAPACITY: return "capacity exceeded";
    }
    return "unknown status";
}

fedd_status fedd_last_error(const fedd_assembler *h, char *buf, size_t len) {
    if (!buf || len == 0) return FEDD_ERR_ARG;
    std::strncpy(buf, h ? h->err.c_str() : thread_error().c_str(), len - 1);
    buf[len - 1] = 0;
    return FEDD_OK;
}

fedd_status fedd_create(const fedd_mesh *mesh, const fedd_params *params, int device, fedd_assembler **out) {
    if (!mesh || !params || !out) return FEDD_ERR_ARG;
    *out = nullptr;
    if (mesh->num_elements <= 0 || mesh->num_nodes <= 0 || !mesh->coords || !mesh->elements) return FEDD_ERR_ARG;
    if (mesh->fe_order != 1 && mesh->fe_order != 2) return FEDD_ERR_ARG;
    if (mesh->num_elements >= (1LL << 28) || mesh->num_nodes >= (1LL << 31)) return FEDD_ERR_ARG;
    const int prob = params->problem;
    if (prob < FEDD_LAPLACE || prob > FEDD_NONLINEAR_ELASTICITY2) return FEDD_ERR_ARG;
    if (prob != FEDD_LAPLACE && mesh->fe_order != 2) return FEDD_ERR_UNSUPPORTED;
    if (prob == FEDD_NAVIER_STOKES && (!mesh->elements_p || mesh->num_nodes_p <= 0)) return FEDD_ERR_ARG;
    if (params->linearization < 0 || params->linearization > 2) return FEDD_ERR_ARG;
    fedd_assembler *h = new (std::nothrow) fedd_assembler;
    if (!h) return FEDD_ERR_NOMEM;
    fedd_status st = guarded(h, [&] {
        FEDD_CUDA(cudaSetDevice(device));
        h->device = device;
        h->prm = *params;
        // 2: FEDDLib's assembleMode "FixedPoint" (the fixed-point matrix);
        // the kernels see the FixedPoint linearization
        h->fp_matrix = params->linearization == 2;
        h->prm.linearization = params->linearization == 1 ? 1 : 0;
        h->order = mesh->fe_order;
        h->npe = h->order == 1 ? 4 : 10;
        h->nn = mesh->num_nodes;
        h->ne = mesh->num_elements;
        cudaStream_t s = 0;
        h->d_err.alloc(1);
        h->d_err.zero(s);
        // device-resident meshes are copied and transposed on the device
        const bool dev_mesh = mesh->flags & FEDD_MESH_DEVICE;
        auto load_conn = [&](DBuf<int32_t> &dst, const int32_t *src, int npe) {
            if (dev_mesh) {
                dst.alloc((size_t)h->ne * npe);
                device_aos_to_soa(src, h->ne, npe, dst.p, s);
            } else {
                std::vector<int32_t> soa = to_soa(src, h->ne, npe);
                dst.upload(soa.data(), soa.size(), s);
            }
        };
        if (dev_mesh) {
            h->xyz.alloc((size_t)h->nn * 3);
            FEDD_CUDA(cudaMemcpyAsync(h->xyz.p, mesh->coords, (size_t)h->nn * 3 * sizeof(double),
                                      cudaMemcpyDeviceToDevice, s));
        } else {
            h->xyz.upload(mesh->coords, (size_t)h->nn * 3, s);
        }
        load_conn(h->conn, mesh->elements, h->npe);
        FEDD_CUDA(cudaStreamSynchronize(s));
        build_graph(h->g, h->ne, h->conn.p, h->npe, h->nn, h->conn.p, h->npe, h->nn, 0, h->d_err.p, s);
        if (prob == FEDD_LAPLACE) {
            build_csr(h->csr[0], h->g.adj_ptr, h->g.adj, h->nn, h->nn, 1, 1, s);
            h->stage_d.alloc((size_t)h->ne * (h->order == 1 ? kLapStrideP1 : kLapStrideP2));
            std::vector<double> t;
            lap_make_tables(h->order, t);
            h->lap_tab.upload(t.data(), t.size(), s);
        } else if (prob == FEDD_NAVIER_STOKES) {
            h->nn_p = mesh->num_nodes_p;
            load_conn(h->conn_p, mesh->elements_p, 4);
            FEDD_CUDA(cudaStreamSynchronize(s));
            build_graph_extra(h->g, h->ne, h->conn_p.p, 4, h->nn_p, 10, h->padj_ptr, h->padj, h->max_padj, h->n_padj,
                              h->d_err.p, s);
            build_graph(h->gp, h->ne, h->conn_p.p, 4, h->nn_p, h->conn.p, 10, h->nn, 0, h->d_err.p, s);
            build_csr(h->csr[0], h->g.adj_ptr, h->g.adj, h->nn, h->nn, 3, 3, s);
            build_csr(h->csr[1], h->padj_ptr, h->padj, h->nn, h->nn_p, 3, 1, s);
            build_csr(h->csr[2], h->gp.adj_ptr, h->gp.adj, h->nn_p, h->nn, 1, 3, s);
            h->ns_fused = build_vertex_map(h->conn.p, h->conn_p.p, h->ne, h->nn, h->nn_p, h->g, h->gp, h->vmap, s);
            h->ninfo.alloc(h->nn);
            launch_ns_node_info(h->g, h->padj_ptr.p, h->ns_fused ? h->vmap.p : nullptr, h->ninfo.p, s);
            // block (1,1): P1-P1 entries are all zero and FEDDLib inserts only
            // |v| > 1e-13 (FE_def.hpp:1024), so the block is empty
            h->csr[3].nrows = h->nn_p;
            h->csr[3].ncols = h->nn_p;
            h->csr[3].nnz = 0;
            h->csr[3].rowptr.alloc(h->nn_p + 1);
            h->csr[3].rowptr.zero(s);
            h->stage_f.alloc((size_t)h->ne * kNSRecord);
            h->work.alloc(1);
            NSTables tabs;
            make_ns_tables(&tabs);
            ns_upload_tables(tabs, &h->ns_tab);
        } else {
            build_csr(h->csr[0], h->g.adj_ptr, h->g.adj, h->nn, h->nn, 3, 3, s);
            h->stage_f.alloc((size_t)h->ne * kElemStride);
            int nq = quad_points(h);
            if (nq != 4 && nq != 5) FEDD_FAIL(FEDD_ERR_UNSUPPORTED, "hyperelastic rules: 4 or 5 points");
            make_hyper_tables(nq, &h->htab);
            set_law(h);
            if (prob == FEDD_ANISO_FIBER) {
                h->qp_inv.alloc((size_t)h->ne * nq * 4);
                h->qp_der.alloc((size_t)h->ne * nq);
                h->qp_fb.alloc((size_t)h->ne * nq);
                h->d_fb.alloc(1);
            }
        }
        FEDD_CUDA(cudaStreamSynchronize(s));
    });
    if (st != FEDD_OK) {
        // keep the handle so the caller can read the message, unless it failed early
        *out = h;
        return st;
    }
    *out = h;
    return FEDD_OK;
}

fedd_status fedd_destroy(fedd_assembler *h) {
    if (!h) return FEDD_ERR_ARG;
    cudaSetDevice(h->device);
    delete h;
    return FEDD_OK;
}

fedd_status fedd_block_info(const fedd_assembler *h, int block, int64_t *nrows, int64_t *ncols, int64_t *nnz) {
    if (!h || block < 0 || block > 3) return FEDD_ERR_ARG;
    if (h->prm.problem != FEDD_NAVIER_STOKES && block != 0) return FEDD_ERR_ARG;
    if (nrows) *nrows = h->csr[block].nrows;
    if (ncols) *ncols = h->csr[block].ncols;
    if (nnz) *nnz = h->csr[block].nnz;
    return FEDD_OK;
}

fedd_status fedd_residual_sizes(const fedd_assembler *h, int64_t *n_u, int64_t *n_p) {
    if (!h) return FEDD_ERR_ARG;
    int dofs = h->prm.problem == FEDD_LAPLACE ? 1 : 3;
    if (n_u) *n_u = h->nn * dofs;
    if (n_p) *n_p = h->prm.problem == FEDD_NAVIER_STOKES ? h->nn_p : 0;
    return FEDD_OK;
}

fedd_status fedd_get_pattern(fedd_assembler *h, int block, int64_t *rowptr_host, int32_t *colind_host) {
    if (!h || block < 0 || block > 3 || !rowptr_host) return FEDD_ERR_ARG;
    if (h->prm.problem != FEDD_NAVIER_STOKES && block != 0) return FEDD_ERR_ARG;
    return guarded(h, [&] {
        FEDD_CUDA(cudaSetDevice(h->device));
        const Csr &c = h->csr[block];
        FEDD_CUDA(cudaMemcpy(rowptr_host, c.rowptr.p, (c.nrows + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost));
        if (c.nnz && colind_host)
            FEDD_CUDA(cudaMemcpy(colind_host, c.colind.p, c.nnz * sizeof(int32_t), cudaMemcpyDeviceToHost));
    });
}

fedd_status fedd_device_pattern(fedd_assembler *h, int block, const int64_t **d_rowptr, const int32_t **d_colind) {
    if (!h || block < 0 || block > 3) return FEDD_ERR_ARG;
    if (h->prm.problem != FEDD_NAVIER_STOKES && block != 0) return FEDD_ERR_ARG;
    if (d_rowptr) *d_rowptr = h->csr[block].rowptr.p;
    if (d_colind) *d_colind = h->csr[block].colind.p;
    return FEDD_OK;
}

fedd_status fedd_assemble_device(fedd_assembler *h, unsigned what, const double *d_u, const double *d_p,
                                 double *d_vals00, double *d_vals01, double *d_vals10, double *d_res_u, double *d_res_p,
                                 void *stream) {
    if (!h || (what & ~(FEDD_JACOBIAN | FEDD_RESIDUAL)) || !what) return FEDD_ERR_ARG;
    const int prob = h->prm.problem;
    if ((what & FEDD_JACOBIAN) && !d_vals00) return FEDD_ERR_ARG;
    if (prob == FEDD_NAVIER_STOKES) {
        if (!d_u) return FEDD_ERR_ARG;
        if ((what & FEDD_JACOBIAN) && (!d_vals01 || !d_vals10)) return FEDD_ERR_ARG;
        if ((what & FEDD_RESIDUAL) && (!d_res_u || !d_res_p)) return FEDD_ERR_ARG;
    } else if (what & FEDD_RESIDUAL) {
        if (!d_res_u) return FEDD_ERR_ARG;
    }
    if ((prob == FEDD_NONLINEAR_ELASTICITY || prob == FEDD_NONLINEAR_ELASTICITY2) && !d_u) return FEDD_ERR_ARG;
    return guarded(h, [&] {
        FEDD_CUDA(cudaSetDevice(h->device));
        run(h, what, d_u, d_p, d_vals00, d_vals01, d_vals10, d_res_u, d_res_p, (cudaStream_t)stream);
    });
}

}  // extern "C"

namespace {

// Host-buffer assembly with the device-to-host copies overlapped: the row
// stage runs in kChunks node ranges on `s`, and after each range its CSR rows
// and residual entries are copied to the host on a second stream while the
// next range is computed (the copy link, about 190 GB/s, bounds this path).
// Navier-Stokes (Newtonian) and the elasticity problems; returns false when
// the plain path has to be taken.
bool run_host_pipelined(fedd_assembler *h, unsigned what, const double *du, const double *dp, double *const *dv,
                        double *dru, double *drp, double *const *hv, double *res_u, double *res_p, cudaStream_t s) {
    const int prob = h->prm.problem;
    const bool ns = prob == FEDD_NAVIER_STOKES;
    const bool hyper = prob == FEDD_LINEAR_ELASTICITY || prob == FEDD_NONLINEAR_ELASTICITY ||
                       prob == FEDD_NONLINEAR_ELASTICITY2 || prob == FEDD_ANISO_FIBER;
    const bool jac = what & FEDD_JACOBIAN, res = what & FEDD_RESIDUAL;
    if (!jac || h->prof || !(hyper || ns)) return false;
    constexpr int K = fedd_assembler::kChunks;
    if (!h->chunks_ready) {
        FEDD_CUDA(cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking));
        for (auto &e : h->chunk_ev) FEDD_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        for (int k = 0; k <= K; k++) {
            h->cut[k] = h->nn * k / K;
            FEDD_CUDA(cudaMemcpy(&h->off00[k], h->csr[0].rowptr.p + 3 * h->cut[k], sizeof(int64_t),
                                 cudaMemcpyDeviceToHost));
            if (ns)
                FEDD_CUDA(cudaMemcpy(&h->off01[k], h->csr[1].rowptr.p + 3 * h->cut[k], sizeof(int64_t),
                                     cudaMemcpyDeviceToHost));
        }
        // element chunk k ends past the largest element any node of chunks
        // 0..k is incident to (a numbering without locality puts every
        // element in chunk 0)
        int64_t mx[K];
        node_range_max_elem(h->g, h->cut, K, mx, 0);
        h->ecut[0] = 0;
        for (int k = 0; k < K; k++) h->ecut[k + 1] = std::max(h->ecut[k], mx[k] + 1);
        h->ecut[K] = h->ne;
        h->chunks_ready = true;
    }
    LaunchCounter lc;
    cudaStream_t cs = h->copy_stream;
    FEDD_CUDA(cudaMemsetAsync(h->d_err.p, 0, sizeof(int), s));
    // a generalized-Newtonian fluid: no Newtonian Laplacian in NA; its
    // viscous element stage runs in the element chunks, folded into the
    // velocity rows.  So do the surrogate's per-point stages.
    const float vd_ns = h->gn_on ? 0.0f : (float)(h->prm.viscosity * h->prm.density);
    const bool mlp = hyper && h->law.kind == kLawMLP;
    const QPDerivs *qpd = nullptr;
    const uint8_t *qfb = nullptr;
    const int nq = h->htab.nq;
    if (mlp) {
        if (!h->has_mlp) FEDD_FAIL(FEDD_ERR_STATE, "surrogate requested but no network set (fedd_set_surrogate)");
        FEDD_CUDA(cudaMemsetAsync(h->d_fb.p, 0, sizeof(int), s));
        qpd = h->qp_der.p;
        qfb = h->qp_fb.p;
        h->last_nqp = h->ne * nq;
    }
    for (int k = 0; k < K; k++) {
        const int64_t n0 = h->cut[k], n1 = h->cut[k + 1], e0 = h->ecut[k], e1 = h->ecut[k + 1];
        if (ns) {
            launch_ns_record(h->xyz.p, h->conn.p, h->conn_p.p, h->ne, du, dp, h->ns_tab, vd_ns, (float)h->prm.density,
                             h->stage_f.p, h->d_err.p, s, lc, e0, e1);
            if (h->gn_on)
                launch_gn_elem(h->xyz.p, h->conn.p, h->ne, du, h->gn, h->prm.linearization, h->stage_gn.p, h->d_err.p,
                               s, lc, e0, e1, h->outflow());
        } else {
            if (mlp && e1 > e0) {  // the points of elements [e0, e1): QPs [e0 nq, e1 nq)
                launch_hyper_invariants(h->xyz.p, h->conn.p, h->ne, du, h->law, h->htab, h->qp_inv.p, h->d_err.p, s,
                                        lc, e0, e1);
                launch_mlp_qp(h->mlp, h->law, h->qp_inv.p + 4 * e0 * nq, (e1 - e0) * nq, h->qp_der.p + e0 * nq,
                              h->qp_fb.p + e0 * nq, h->d_fb.p, h->d_err.p, s, lc);
            }
            launch_hyper_elem(h->xyz.p, h->conn.p, h->ne, du, h->law, h->htab, qpd, qfb, h->stage_f.p,
                              res && du != nullptr, h->d_err.p, s, lc, e0, e1);
        }
        if (ns) {
            launch_ns_vel_rows(h->g, h->ninfo.p, h->stage_f.p, h->ns_tab, h->csr[0].rowptr.p, h->csr[1].rowptr.p,
                               dv[0], dv[1], res ? dru : nullptr, vd_ns, (float)h->prm.density, h->prm.linearization,
                               1, h->g.max_adj, h->max_padj, h->ns_fused ? h->vmap.p : nullptr, h->csr[2].rowptr.p,
                               dv[2], res ? drp : nullptr, h->gn_on ? h->stage_gn.p : nullptr, s, lc, n0, n1,
                               nullptr, h->coeff);
        } else
            launch_hyper_rows(h->g, h->stage_f.p, h->csr[0].rowptr.p, dv[0], res ? dru : nullptr, n1, s, lc, n0);
        FEDD_CUDA(cudaEventRecord(h->chunk_ev[k], s));
        FEDD_CUDA(cudaStreamWaitEvent(cs, h->chunk_ev[k], 0));
        const int64_t a0 = h->off00[k], a1 = h->off00[k + 1];
        if (a1 > a0)
            FEDD_CUDA(cudaMemcpyAsync(hv[0] + a0, dv[0] + a0, (a1 - a0) * sizeof(double), cudaMemcpyDeviceToHost, cs));
        if (ns && h->off01[k + 1] > h->off01[k])
            FEDD_CUDA(cudaMemcpyAsync(hv[1] + h->off01[k], dv[1] + h->off01[k],
                                      (h->off01[k + 1] - h->off01[k]) * sizeof(double), cudaMemcpyDeviceToHost, cs));
        if (res && n1 > n0)
            FEDD_CUDA(cudaMemcpyAsync(res_u + 3 * n0, dru + 3 * n0, 3 * (n1 - n0) * sizeof(double),
                                      cudaMemcpyDeviceToHost, cs));
    }
    if (ns) {
        if (!h->ns_fused)
            launch_ns_pres_rows(h->gp, h->stage_f.p, h->ns_tab, h->csr[2].rowptr.p, dv[2], res ? drp : nullptr, 1,
                                h->gp.max_adj, s, lc, h->coeff);
        FEDD_CUDA(cudaEventRecord(h->chunk_ev[K], s));
        FEDD_CUDA(cudaStreamWaitEvent(cs, h->chunk_ev[K], 0));
        if (h->csr[2].nnz)
            FEDD_CUDA(cudaMemcpyAsync(hv[2], dv[2], h->csr[2].nnz * sizeof(double), cudaMemcpyDeviceToHost, cs));
        if (res) FEDD_CUDA(cudaMemcpyAsync(res_p, drp, h->nn_p * sizeof(double), cudaMemcpyDeviceToHost, cs));
    }
    FEDD_CUDA(cudaEventRecord(h->chunk_ev[K + 1], cs));
    FEDD_CUDA(cudaStreamWaitEvent(s, h->chunk_ev[K + 1], 0));
    h->launches = lc.n;
    return true;
}

}  // namespace

extern "C" {

fedd_status fedd_assemble(fedd_assembler *h, unsigned what, const double *u, const double *p, double *vals00,
                          double *vals01, double *vals10, double *res_u, double *res_p, void *stream) {
    if (!h || !what || (what & ~(FEDD_JACOBIAN | FEDD_RESIDUAL))) return FEDD_ERR_ARG;
    const int prob = h->prm.problem;
    if ((what & FEDD_JACOBIAN) && !vals00) return FEDD_ERR_ARG;
    if (prob == FEDD_NAVIER_STOKES && (!u || ((what & FEDD_JACOBIAN) && (!vals01 || !vals10)) ||
                                       ((what & FEDD_RESIDUAL) && (!res_u || !res_p))))
        return FEDD_ERR_ARG;
    if (prob != FEDD_NAVIER_STOKES && (what & FEDD_RESIDUAL) && !res_u) return FEDD_ERR_ARG;
    if ((prob == FEDD_NONLINEAR_ELASTICITY || prob == FEDD_NONLINEAR_ELASTICITY2) && !u) return FEDD_ERR_ARG;
    return guarded(h, [&] {
        FEDD_CUDA(cudaSetDevice(h->device));
        cudaStream_t s = (cudaStream_t)stream;
        const int dofs = prob == FEDD_LAPLACE ? 1 : 3;
        const bool jac = what & FEDD_JACOBIAN, res = what & FEDD_RESIDUAL;
        const double *du = nullptr, *dp = nullptr;
        if (u && prob != FEDD_LAPLACE) {
            if (h->u_dev.n != (size_t)(h->nn * dofs)) h->u_dev.alloc(h->nn * dofs);
            FEDD_CUDA(cudaMemcpyAsync(h->u_dev.p, u, h->nn * dofs * sizeof(double), cudaMemcpyHostToDevice, s));
            du = h->u_dev.p;
        }
        if (prob == FEDD_NAVIER_STOKES && p) {
            if (h->p_dev.n != (size_t)h->nn_p) h->p_dev.alloc(h->nn_p);
            FEDD_CUDA(cudaMemcpyAsync(h->p_dev.p, p, h->nn_p * sizeof(double), cudaMemcpyHostToDevice, s));
            dp = h->p_dev.p;
        }
        double *dv[3] = {nullptr, nullptr, nullptr};
        const int nblk = prob == FEDD_NAVIER_STOKES ? 3 : 1;
        if (jac)
            for (int b = 0; b < nblk; b++) {
                if (h->v_dev[b].n != (size_t)h->csr[b].nnz) h->v_dev[b].alloc(h->csr[b].nnz);
                dv[b] = h->v_dev[b].p;
            }
        double *dru = nullptr, *drp = nullptr;
        if (res) {
            if (h->ru_dev.n != (size_t)(h->nn * dofs)) h->ru_dev.alloc(h->nn * dofs);
            dru = h->ru_dev.p;
            if (prob == FEDD_NAVIER_STOKES) {
                if (h->rp_dev.n != (size_t)h->nn_p) h->rp_dev.alloc(h->nn_p);
                drp = h->rp_dev.p;
            }
        }
        double *hv[3] = {vals00, vals01, vals10};
        if (run_host_pipelined(h, what, du, dp, dv, dru, drp, hv, res_u, res_p, s)) {
            read_dev_error(h, s);
            return;
        }
        run(h, what, du, dp, dv[0], dv[1], dv[2], dru, drp, s);
        if (jac)
            for (int b = 0; b < nblk; b++)
                if (h->csr[b].nnz)
                    FEDD_CUDA(cudaMemcpyAsync(hv[b], dv[b], h->csr[b].nnz * sizeof(double), cudaMemcpyDeviceToHost, s));
        if (res) {
            FEDD_CUDA(cudaMemcpyAsync(res_u, dru, h->nn * dofs * sizeof(double), cudaMemcpyDeviceToHost, s));
            if (drp) FEDD_CUDA(cudaMemcpyAsync(res_p, drp, h->nn_p * sizeof(double), cudaMemcpyDeviceToHost, s));
        }
        read_dev_error(h, s);
    });
}

fedd_status fedd_check(fedd_assembler *h, void *stream) {
    if (!h) return FEDD_ERR_ARG;
    return guarded(h, [&] {
        FEDD_CUDA(cudaSetDevice(h->device));
        read_dev_error(h, (cudaStream_t)stream);
    });
}

fedd_status fedd_launch_count(const fedd_assembler *h, int64_t *launches) {
    if (!h || !launches) return FEDD_ERR_ARG;
    *launches = h->launches;
    return FEDD_OK;
}

fedd_status fedd_set_profiling(fedd_assembler *h, int on) {
    if (!h) return FEDD_ERR_ARG;
    return guarded(h, [&] {
        FEDD_CUDA(cudaSetDevice(h->device));
        if (on && h->ev.empty()) {
            h->ev.resize((size_t)fedd_assembler::kProfCalls * fedd_assembler::kProfStages * 2);
            for (auto &e : h->ev) FEDD_CUDA(cudaEventCreate(&e));
        }
        h->prof = on != 0;
        h->prof_calls = 0;
        h->prof_stage = 0;
    });
}

fedd_status fedd_stage_times(fedd_assembler *h, int max_stages, double *ms_total, int *nstages, int64_t *calls) {
    if (!h || !ms_total || !nstages || !calls || max_stages <= 0) return FEDD_ERR_ARG;
    return guarded(h, [&] {
        FEDD_CUDA(cudaSetDevice(h->device));
        const int ns = std::min<int>((int)h->stage_names.size(), max_stages);
        for (int k = 0; k < ns; k++) ms_total[k] = 0.0;
        for (int c = 0; c < h->prof_calls; c++)
            for (int k = 0; k < ns; k++) {
                cudaEvent_t *e = &h->ev[((size_t)c * fedd_assembler::kProfStages + k) * 2];
                FEDD_CUDA(cudaEventSynchronize(e[1]));
                float ms = 0.0f;
                FEDD_CUDA(cudaEventElapsedTime(&ms, e[0], e[1]));
                ms_total[k] += ms;
            }
        *nstages = ns;
        *calls = h->prof_calls;
        h->prof_calls = 0;
    });
}

const char *fedd_stage_name(const fedd_assembler *h, int stage) {
    if (!h || stage < 0 || stage >= (int)h->stage_names.size()) return "";
    return h->stage_names[stage].c_str();
}

fedd_status fedd_element_matrices(fedd_assembler *h, const double *u, const double *p, int64_t first, int64_t count,
                                  double *Ke, double *re) {
    if (!h || !Ke || !re || first < 0 || count < 0 || first + count > h->ne) return FEDD_ERR_ARG;
    const int prob = h->prm.problem;
    if ((prob == FEDD_NAVIER_STOKES || prob == FEDD_NONLINEAR_ELASTICITY || prob == FEDD_NONLINEAR_ELASTICITY2) && !u)
        return FEDD_ERR_ARG;
    return guarded(h, [&] {
        FEDD_CUDA(cudaSetDevice(h->device));
        cudaStream_t s = 0;
        const int dofs = prob == FEDD_LAPLACE ? 1 : 3;
        const double *du = nullptr, *dp = nullptr;
        DBuf<double> tu, tp, tK, tr;
        if (u && prob != FEDD_LAPLACE) {
            tu.upload(u, h->nn * dofs, s);
            du = tu.p;
        }
        if (prob == FEDD_NAVIER_STOKES && p) {
            tp.upload(p, h->nn_p, s);
            dp = tp.p;
        }
        LaunchCounter lc;
        FEDD_CUDA(cudaMemsetAsync(h->d_err.p, 0, sizeof(int), s));
        int nd = 0;
        if (prob == FEDD_LAPLACE) {
            nd = h->npe;
            launch_lap_elem(h->xyz.p, h->conn.p, h->ne, h->order, h->lap_tab.p, h->prm.source, h->stage_d.p,
                            h->d_err.p, s, lc);
        } else if (prob == FEDD_NAVIER_STOKES) {
            nd = 34;
            launch_ns_record(h->xyz.p, h->conn.p, h->conn_p.p, h->ne, du, dp, h->ns_tab,
                             h->gn_on ? 0.0f : (float)(h->prm.viscosity * h->prm.density), (float)h->prm.density,
                             h->stage_f.p, h->d_err.p, s, lc);
            if (h->gn_on)
                launch_gn_elem(h->xyz.p, h->conn.p, h->ne, du, h->gn, h->prm.linearization, h->stage_gn.p, h->d_err.p,
                               s, lc, 0, -1, h->outflow());
        } else {
            nd = 30;
            const QPDerivs *qpd = nullptr;
            const uint8_t *qfb = nullptr;
            if (h->law.kind == kLawMLP) {
                if (!h->has_mlp) FEDD_FAIL(FEDD_ERR_STATE, "surrogate requested but no network set");
                launch_hyper_invariants(h->xyz.p, h->conn.p, h->ne, du, h->law, h->htab, h->qp_inv.p, h->d_err.p, s,
                                        lc);
                FEDD_CUDA(cudaMemsetAsync(h->d_fb.p, 0, sizeof(int), s));
                launch_mlp_qp(h->mlp, h->law, h->qp_inv.p, h->ne * h->htab.nq, h->qp_der.p, h->qp_fb.p, h->d_fb.p, h->d_err.p, s,
                              lc);
                qpd = h->qp_der.p;
                qfb = h->qp_fb.p;
            }
            launch_hyper_elem(h->xyz.p, h->conn.p, h->ne, du, h->law, h->htab, qpd, qfb, h->stage_f.p, du != nullptr,
                              h->d_err.p, s, lc);
        }
        if (count == 0) return;
        tK.alloc((size_t)count * nd * nd);
        tr.alloc((size_t)count * nd);
        if (prob == FEDD_LAPLACE)
            launch_lap_dense(h->stage_d.p, h->order, first, count, tK.p, tr.p, s);
        else if (prob == FEDD_NAVIER_STOKES) {
            launch_ns_dense(h->stage_f.p, h->ns_tab, first, count,
                            h->gn_on ? 0.0f : (float)(h->prm.viscosity * h->prm.density), (float)h->prm.density,
                            h->prm.linearization, tK.p, tr.p, s, h->coeff);
            if (h->gn_on) launch_gn_dense(h->stage_gn.p, first, count, tK.p, tr.p, s, h->coeff.uu);
        } else
            launch_hyper_dense(h->stage_f.p, first, count, tK.p, tr.p, s);
        FEDD_CUDA(cudaMemcpyAsync(Ke, tK.p, (size_t)count * nd * nd * sizeof(double), cudaMemcpyDeviceToHost, s));
        FEDD_CUDA(cudaMemcpyAsync(re, tr.p, (size_t)count * nd * sizeof(double), cudaMemcpyDeviceToHost, s));
        read_dev_error(h, s);
    });
}

fedd_status fedd_set_surrogate(fedd_assembler *h, const fedd_mlp_desc *m) {
    if (!h || !m) return FEDD_ERR_ARG;
    if (h->prm.problem != FEDD_ANISO_FIBER) return FEDD_ERR_STATE;
    const int H = m->hidden;
    if (H < 16 || H > 128 || H % 16 || !m->W1 || !m->b1 || !m->W2 || !m->b2 || !m->w3) return FEDD_ERR_ARG;
    return guarded(h, [&] {
        if (m->in_clamp & ~0xF) FEDD_FAIL(FEDD_ERR_ARG, "in_clamp: bits 0-3 only (one per input)");
        FEDD_CUDA(cudaSetDevice(h->device));
        auto bf = [](const float *x, size_t n) {
            std::vector<__nv_bfloat16> v(n);
            for (size_t i = 0; i < n; i++) v[i] = __float2bfloat16_rn(x[i]);
            return v;
        };
        auto w1 = bf(m->W1, (size_t)H * 4), w2 = bf(m->W2, (size_t)H * H), w3 = bf(m->w3, (size_t)H);
        h->mW1.upload(w1.data(), w1.size());
        h->mW2.upload(w2.data(), w2.size());
        h->mw3.upload(w3.data(), w3.size());
        h->mb1.upload(m->b1, H);
        h->mb2.upload(m->b2, H);
        MLPDev d{};
        d.hidden = H;
        d.W1 = h->mW1.p; d.W2 = h->mW2.p; d.w3 = h->mw3.p;
        d.b1 = h->mb1.p; d.b2 = h->mb2.p;
        d.b3 = m->b3; d.out_scale = m->out_scale;
        d.in_clamp = m->in_clamp;
        for (int k = 0; k < 4; k++) {
            d.in_shift[k] = m->in_shift[k]; d.in_scale[k] = m->in_scale[k];
            d.inv_lo[k] = m->inv_lo[k]; d.inv_hi[k] = m->inv_hi[k];
        }
        if (H == 64) {
            MlpConst &c = d.c;
            c.nact = 0;
            for (int k = 0; k < 4; k++)
                if (m->in_scale[k] != 0.0f) c.act[c.nact++] = k;
            for (int i = 0; i < 64; i++) {
                for (int k = 0; k < 4; k++) c.W1[i][k] = __bfloat162float(w1[4 * i + k]);
                for (int a = 0; a < 4; a++) c.Wact[a][i] = a < c.nact ? c.W1[i][c.act[a]] : 0.0f;
                c.b1[i] = m->b1[i];
                c.b2[i] = m->b2[i];
                c.w3[i] = __bfloat162float(w3[i]);
            }
        }
        h->mlp = d;
        // frozen I1 and J inputs: the element kernel takes the fibre-block path
        h->law.mlp_fibre = (m->in_scale[0] == 0.0f && m->in_scale[1] == 0.0f) ? 1 : 0;
        h->has_mlp = true;
        FEDD_CUDA(cudaDeviceSynchronize());
    });
}

fedd_status fedd_surrogate_fallbacks(fedd_assembler *h, int64_t *count, int64_t *total) {
    if (!h || !count || !total) return FEDD_ERR_ARG;
    if (h->prm.problem != FEDD_ANISO_FIBER || h->law.kind != kLawMLP) return FEDD_ERR_STATE;
    return guarded(h, [&] {
        FEDD_CUDA(cudaSetDevice(h->device));
        int c = 0;
        FEDD_CUDA(cudaMemcpy(&c, h->d_fb.p, sizeof c, cudaMemcpyDeviceToHost));
        *count = c;
        *total = h->last_nqp;
    });
}

fedd_status fedd_qp_invariants(fedd_assembler *h, const double *u, float *out) {
    if (!h || !u || !out) return FEDD_ERR_ARG;
    if (h->prm.problem == FEDD_LAPLACE || h->prm.problem == FEDD_NAVIER_STOKES) return FEDD_ERR_STATE;
    return guarded(h, [&] {
        FEDD_CUDA(cudaSetDevice(h->device));
        cudaStream_t s = 0;
        DBuf<double> du;
        DBuf<float> inv;
        du.upload(u, (size_t)h->nn * 3, s);
        inv.alloc((size_t)h->ne * h->htab.nq * 4);
        LaunchCounter lc;
        FEDD_CUDA(cudaMemsetAsync(h->d_err.p, 0, sizeof(int), s));
        launch_hyper_invariants(h->xyz.p, h->conn.p, h->ne, du.p, h->law, h->htab, inv.p, h->d_err.p, s, lc);
        FEDD_CUDA(cudaMemcpyAsync(out, inv.p, inv.n * sizeof(float), cudaMemcpyDeviceToHost, s));
        read_dev_error(h, s);
    });
}

fedd_status fedd_set_viscosity_law(fedd_assembler *h, int32_t model, const double *prm, double gamma_min) {
    if (!h) return FEDD_ERR_ARG;
    if (h->prm.problem != FEDD_NAVIER_STOKES) return FEDD_ERR_STATE;
    if (model < 0) {
        h->gn_on = false;
        return FEDD_OK;
    }
    if (model > 2 || !prm) return FEDD_ERR_ARG;
    return guarded(h, [&] {
        FEDD_CUDA(cudaSetDevice(h->device));
        ViscLaw L{};
        L.model = model;
        for (int k = 0; k < 5; k++) L.prm[k] = (float)prm[k];
        L.gamma_min = (float)gamma_min;
        if (h->stage_gn.n < (size_t)h->ne * kGNStride) h->stage_gn.alloc((size_t)h->ne * kGNStride);
        h->gn = L;
        h->gn_on = true;
    });
}

fedd_status fedd_set_element_moduli(fedd_assembler *h, const double *E) {
    if (!h) return FEDD_ERR_ARG;
    const int pb = h->prm.problem;
    if (pb != FEDD_LINEAR_ELASTICITY && pb != FEDD_NONLINEAR_ELASTICITY && pb != FEDD_NONLINEAR_ELASTICITY2)
        return FEDD_ERR_STATE;
    if (E)
        for (int64_t e = 0; e < h->ne; e++)
            if (!std::isfinite(E[e]) || !(E[e] > 0.0)) return FEDD_ERR_ARG;
    return guarded(h, [&] {
        FEDD_CUDA(cudaSetDevice(h->device));
        if (!E) {
            h->emod.release();
        } else {
            std::vector<float> sc((size_t)h->ne);
            for (int64_t e = 0; e < h->ne; e++) sc[(size_t)e] = (float)(E[e] / h->prm.E);
            h->emod.alloc((size_t)h->ne);
            FEDD_CUDA(cudaMemcpy(h->emod.p, sc.data(), sc.size() * sizeof(float), cudaMemcpyHostToDevice));
        }
        h->law.escale = h->emod.n ? h->emod.p : nullptr;
    });
}

fedd_status fedd_set_coeff(fedd_assembler *h, const double coeff[4]) {
    if (!h || !coeff) return FEDD_ERR_ARG;
    if (h->prm.problem != FEDD_NAVIER_STOKES) return FEDD_ERR_STATE;
    for (int k = 0; k < 4; k++)
        if (!std::isfinite(coeff[k])) return FEDD_ERR_ARG;
    h->coeff.uu = coeff[0];
    h->coeff.up = coeff[1];
    h->coeff.pu = coeff[2];
    return FEDD_OK;
}

fedd_status fedd_set_outflow_faces(fedd_assembler *h, const int32_t *faces, int64_t nfaces) {
    if (!h || nfaces < 0 || (nfaces > 0 && !faces)) return FEDD_ERR_ARG;
    if (h->prm.problem != FEDD_NAVIER_STOKES) return FEDD_ERR_STATE;
    return guarded(h, [&] {
        FEDD_CUDA(cudaSetDevice(h->device));
        if (nfaces == 0) {
            h->of_elem.release();
            h->of_face.release();
            h->of_n = 0;
            return;
        }
        // every vertex face of every element, keyed by its sorted vertex ids
        const int64_t ne = h->ne;
        std::vector<int32_t> v((size_t)4 * ne);
        FEDD_CUDA(cudaMemcpy(v.data(), h->conn.p, v.size() * sizeof(int32_t), cudaMemcpyDeviceToHost));
        struct Key {
            int32_t a, b, c;
            bool operator==(const Key &o) const { return a == o.a && b == o.b && c == o.c; }
        };
        struct Hash {
            size_t operator()(const Key &k) const {
                return ((size_t)(uint32_t)k.a * 0x9E3779B97F4A7C15ull) ^ ((size_t)(uint32_t)k.b * 0xC2B2AE3D27D4EB4Full) ^
                       (size_t)(uint32_t)k.c;
            }
        };
        auto key = [](int32_t x, int32_t y, int32_t z) {
            if (x > y) std::swap(x, y);
            if (y > z) std::swap(y, z);
            if (x > y) std::swap(x, y);
            return Key{x, y, z};
        };
        std::unordered_map<Key, int64_t, Hash> owner;  // element, or -2 where two elements share the face
        owner.reserve((size_t)4 * ne);
        static const int FV[4][3] = {{0, 1, 2}, {0, 1, 3}, {0, 2, 3}, {1, 2, 3}};
        for (int64_t e = 0; e < ne; e++)
            for (int f = 0; f < 4; f++) {
                const Key k = key(v[(size_t)FV[f][0] * ne + e], v[(size_t)FV[f][1] * ne + e], v[(size_t)FV[f][2] * ne + e]);
                auto it = owner.find(k);
                if (it == owner.end())
                    owner.emplace(k, e);
                else
                    it->second = -2;
            }
        // per element the last face listed for it (the reference keeps the
        // surface data of an element's last flagged sub-element)
        std::vector<int64_t> taken((size_t)ne, -1);
        for (int64_t i = 0; i < nfaces; i++) {
            const int32_t *f = faces + 3 * i;
            for (int t = 0; t < 3; t++)
                if (f[t] < 0 || f[t] >= h->nn) FEDD_FAIL(FEDD_ERR_ARG, "outflow face " + std::to_string(i) + ": node out of range");
            auto it = owner.find(key(f[0], f[1], f[2]));
            if (it == owner.end()) FEDD_FAIL(FEDD_ERR_ARG, "outflow face " + std::to_string(i) + " is no face of any element");
            if (it->second < 0)
                FEDD_FAIL(FEDD_ERR_ARG, "outflow face " + std::to_string(i) + " is shared by two elements (not a boundary face)");
            taken[(size_t)it->second] = i;
        }
        std::vector<int32_t> el, fc;
        for (int64_t e = 0; e < ne; e++)
            if (taken[(size_t)e] >= 0) {
                el.push_back((int32_t)e);
                for (int t = 0; t < 3; t++) fc.push_back(faces[3 * taken[(size_t)e] + t]);
            }
        h->of_elem.upload(el.data(), el.size());
        h->of_face.upload(fc.data(), fc.size());
        h->of_n = (int64_t)el.size();
        FEDD_CUDA(cudaDeviceSynchronize());
    });
}

fedd_status fedd_dirichlet_set(fedd_assembler *h, const uint8_t *mask_u, const uint8_t *mask_p) {
    if (!h) return FEDD_ERR_ARG;
    if (mask_p && h->prm.problem != FEDD_NAVIER_STOKES) return FEDD_ERR_ARG;
    return guarded(h, [&] {
        FEDD_CUDA(cudaSetDevice(h->device));
        const int64_t n_u = h->csr[0].nrows, n_p = h->prm.problem == FEDD_NAVIER_STOKES ? h->csr[2].nrows : 0;
        std::vector<int64_t> ru, rp;
        for (int64_t k = 0; mask_u && k < n_u; k++)
            if (mask_u[k]) ru.push_back(k);
        for (int64_t k = 0; mask_p && k < n_p; k++)
            if (mask_p[k]) rp.push_back(k);
        h->dir_u.release();
        h->dir_p.release();
        h->n_dir_u = h->n_dir_p = 0;
        if (!ru.empty()) h->dir_u.upload(ru.data(), ru.size(), 0);
        if (!rp.empty()) h->dir_p.upload(rp.data(), rp.size(), 0);
        FEDD_CUDA(cudaStreamSynchronize(0));
        h->n_dir_u = (int64_t)ru.size();
        h->n_dir_p = (int64_t)rp.size();
    });
}

fedd_status fedd_dirichlet_system(fedd_assembler *h, double *d_vals00, double *d_vals01, double *d_vals10,
                                  void *stream) {
    if (!h || !d_vals00) return FEDD_ERR_ARG;
    const bool ns = h->prm.problem == FEDD_NAVIER_STOKES;
    if (ns && (!d_vals01 || !d_vals10)) return FEDD_ERR_ARG;
    return guarded(h, [&] {
        FEDD_CUDA(cudaSetDevice(h->device));
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        LaunchCounter lc;
        launch_dirichlet_rows(h->dir_u.p, h->n_dir_u, h->csr[0].rowptr.p, h->csr[0].colind.p, d_vals00, true, s, lc);
        if (ns) {
            launch_dirichlet_rows(h->dir_u.p, h->n_dir_u, h->csr[1].rowptr.p, h->csr[1].colind.p, d_vals01, false, s,
                                  lc);
            // pressure rows: block (1,0) zero; the (1,1) block of P2-P1 is empty
            launch_dirichlet_rows(h->dir_p.p, h->n_dir_p, h->csr[2].rowptr.p, h->csr[2].colind.p, d_vals10, false, s,
                                  lc);
        }
        h->launches = lc.n;
    });
}

fedd_status fedd_dirichlet_rhs(fedd_assembler *h, const double *d_g_u, const double *d_g_p, const double *d_sub_u,
                               const double *d_sub_p, double *d_res_u, double *d_res_p, void *stream) {
    if (!h || (!d_res_u && !d_res_p)) return FEDD_ERR_ARG;
    return guarded(h, [&] {
        FEDD_CUDA(cudaSetDevice(h->device));
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        LaunchCounter lc;
        if (d_res_u) launch_dirichlet_rhs(h->dir_u.p, h->n_dir_u, d_g_u, d_sub_u, d_res_u, s, lc);
        if (d_res_p) launch_dirichlet_rhs(h->dir_p.p, h->n_dir_p, d_g_p, d_sub_p, d_res_p, s, lc);
        h->launches = lc.n;
    });
}

fedd_status fedd_law_eval(fedd_assembler *h, int64_t n, const double *F, double *psi, double *P, double *A) {
    if (!h || n < 0 || !F || !psi || !P || !A) return FEDD_ERR_ARG;
    if (h->prm.problem == FEDD_LAPLACE || h->prm.problem == FEDD_NAVIER_STOKES) return FEDD_ERR_STATE;
    if (h->law.kind == kLawMLP && !h->has_mlp) return FEDD_ERR_STATE;
    return guarded(h, [&] {
        FEDD_CUDA(cudaSetDevice(h->device));
        DBuf<double> dF, dpsi, dP, dA;
        dF.upload(F, (size_t)n * 9);
        dpsi.alloc(n); dP.alloc((size_t)n * 9); dA.alloc((size_t)n * 81);
        launch_law_eval(h->law, h->law.kind == kLawMLP ? &h->mlp : nullptr, n, dF.p, dpsi.p, dP.p, dA.p, 0);
        FEDD_CUDA(cudaMemcpy(psi, dpsi.p, n * sizeof(double), cudaMemcpyDeviceToHost));
        FEDD_CUDA(cudaMemcpy(P, dP.p, n * 9 * sizeof(double), cudaMemcpyDeviceToHost));
        FEDD_CUDA(cudaMemcpy(A, dA.p, n * 81 * sizeof(double), cudaMemcpyDeviceToHost));
    });
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Element matrices without allocation (fedd_element_matrices_noalloc).
//
// fedd_element_matrices stages its dense output in device buffers it
// allocates and frees on every call.  Some callers cannot allow that: a host
// that keeps other streams of the device busy cannot accept the device-wide
// synchronisation a cudaFree implies, and a host that reserved its device
// memory once at start-up (its own pool) must not see the footprint grow per
// call.  This variant stages the dense output in one file-scope device array
// instead, and runs the element stage over the requested elements only, so
// it makes no allocation at all: no cudaMalloc/cudaFree and no allocating
// library routine.
//
// Limits and rules:
//  * scratch is kNoAllocScratchDoubles doubles (4 MiB) per device; a call
//    needs count * nd * (nd + 1) of them and is rejected with FEDD_ERR_ARG
//    (and a message naming the limit) when that is more;
//  * every call looks up the array's device address with
//    cudaGetSymbolAddress while the handle's device is current (the lookup
//    allocates nothing; doing it per call keeps the address valid across a
//    cudaDeviceReset by the caller); the first call on a device may load
//    the module there, so make it before any stream capture begins;
//  * nothing in the scratch has to start at zero: the dense kernels write
//    every entry they later copy out; the handle's error word, which must
//    start at zero, is cleared by the call itself;
//  * there is one scratch array per device, shared by every handle on it:
//    calls that overlap in time on one device race on it, so callers
//    serialise them.  The call also writes the handle's element stage and
//    error word on its stream, so it must not overlap any other call on the
//    same handle either (the call synchronises its stream before returning);
//  * generalized-Newtonian handles are not supported (their viscous stage is
//    not staged here): FEDD_ERR_UNSUPPORTED with a message.
namespace {

constexpr size_t kNoAllocScratchDoubles = size_t(1) << 19;

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchDoubles];

// Device address of the scratch array on the current device.
double *noalloc_scratch() {
    void *ptr = nullptr;
    const cudaError_t rc = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (rc != cudaSuccess || !ptr)
        FEDD_FAIL(FEDD_ERR_CUDA, std::string("cudaGetSymbolAddress of the element scratch failed: ") +
                                     cudaGetErrorString(rc));
    return static_cast<double *>(ptr);
}

}  // namespace

extern "C" fedd_status fedd_element_matrices_noalloc(fedd_assembler *h, const double *d_u, const double *d_p,
                                                     int64_t first, int64_t count, double *Ke, double *re,
                                                     void *stream) {
    if (!h || !Ke || !re || first < 0 || count < 0 || first + count > h->ne) return FEDD_ERR_ARG;
    const int prob = h->prm.problem;
    if ((prob == FEDD_NAVIER_STOKES || prob == FEDD_NONLINEAR_ELASTICITY || prob == FEDD_NONLINEAR_ELASTICITY2) &&
        !d_u)
        return FEDD_ERR_ARG;
    return guarded(h, [&] {
        if (h->gn_on)
            FEDD_FAIL(FEDD_ERR_UNSUPPORTED, "fedd_element_matrices_noalloc: generalized-Newtonian handles are not "
                                            "supported (use fedd_element_matrices)");
        const int nd = prob == FEDD_LAPLACE ? h->npe : prob == FEDD_NAVIER_STOKES ? 34 : 30;
        const size_t per = (size_t)nd * (nd + 1);
        const int64_t cap = (int64_t)(kNoAllocScratchDoubles / per);
        if (count > cap)
            FEDD_FAIL(FEDD_ERR_ARG, "fedd_element_matrices_noalloc: count " + std::to_string(count) +
                                        " exceeds the static scratch of " +
                                        std::to_string(kNoAllocScratchDoubles * sizeof(double)) + " bytes (at most " +
                                        std::to_string(cap) + " elements of " + std::to_string(nd) + " dofs per call)");
        FEDD_CUDA(cudaSetDevice(h->device));
        double *scratch = noalloc_scratch();
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        const double *du = prob == FEDD_LAPLACE ? nullptr : d_u;
        const double *dp = prob == FEDD_NAVIER_STOKES ? d_p : nullptr;
        const int64_t e0 = first, e1 = first + count;
        LaunchCounter lc;
        FEDD_CUDA(cudaMemsetAsync(h->d_err.p, 0, sizeof(int), s));
        if (count > 0) {
            // the element stage of the requested elements only
            if (prob == FEDD_LAPLACE) {
                launch_lap_elem(h->xyz.p, h->conn.p, h->ne, h->order, h->lap_tab.p, h->prm.source, h->stage_d.p,
                                h->d_err.p, s, lc, e0, e1);
            } else if (prob == FEDD_NAVIER_STOKES) {
                launch_ns_record(h->xyz.p, h->conn.p, h->conn_p.p, h->ne, du, dp, h->ns_tab,
                                 (float)(h->prm.viscosity * h->prm.density), (float)h->prm.density, h->stage_f.p,
                                 h->d_err.p, s, lc, e0, e1);
            } else {
                const QPDerivs *qpd = nullptr;
                const uint8_t *qfb = nullptr;
                if (h->law.kind == kLawMLP) {
                    if (!h->has_mlp) FEDD_FAIL(FEDD_ERR_STATE, "surrogate requested but no network set");
                    const int nq = h->htab.nq;
                    launch_hyper_invariants(h->xyz.p, h->conn.p, h->ne, du, h->law, h->htab, h->qp_inv.p, h->d_err.p,
                                            s, lc, e0, e1);
                    FEDD_CUDA(cudaMemsetAsync(h->d_fb.p, 0, sizeof(int), s));
                    launch_mlp_qp(h->mlp, h->law, h->qp_inv.p + 4 * e0 * nq, count * nq, h->qp_der.p + e0 * nq,
                                  h->qp_fb.p + e0 * nq, h->d_fb.p, h->d_err.p, s, lc);
                    qpd = h->qp_der.p;
                    qfb = h->qp_fb.p;
                }
                launch_hyper_elem(h->xyz.p, h->conn.p, h->ne, du, h->law, h->htab, qpd, qfb, h->stage_f.p,
                                  du != nullptr, h->d_err.p, s, lc, e0, e1);
            }
            double *sK = scratch, *sr = scratch + (size_t)count * nd * nd;
            if (prob == FEDD_LAPLACE)
                launch_lap_dense(h->stage_d.p, h->order, first, count, sK, sr, s);
            else if (prob == FEDD_NAVIER_STOKES)
                launch_ns_dense(h->stage_f.p, h->ns_tab, first, count, (float)(h->prm.viscosity * h->prm.density),
                                (float)h->prm.density, h->prm.linearization, sK, sr, s, h->coeff);
            else
                launch_hyper_dense(h->stage_f.p, first, count, sK, sr, s);
            FEDD_CUDA(cudaMemcpyAsync(Ke, sK, (size_t)count * nd * nd * sizeof(double), cudaMemcpyDeviceToHost, s));
            FEDD_CUDA(cudaMemcpyAsync(re, sr, (size_t)count * nd * sizeof(double), cudaMemcpyDeviceToHost, s));
        }
        read_dev_error(h, s);
    });
}

// ---------------------------------------------------------------------------
// Element geometry as the element kernels use it (fedd_element_geometry).
namespace {

__global__ void k_element_geometry(const double *__restrict__ xyz, const int32_t *__restrict__ conn, int64_t ne,
                                   int64_t first, int64_t count, double *det, float *binv) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= count) return;
    const int64_t e = first + k;
    float Bi[9];
    det[k] = geometry_fp64(xyz, conn[e], conn[ne + e], conn[2 * ne + e], conn[3 * ne + e], Bi);
#pragma unroll
    for (int i = 0; i < 9; i++) binv[9 * k + i] = Bi[i];
}

}  // namespace

extern "C" fedd_status fedd_element_geometry(fedd_assembler *h, int64_t first, int64_t count, double *det,
                                             float *binv) {
    if (!h || !det || !binv || first < 0 || count < 0 || first + count > h->ne) return FEDD_ERR_ARG;
    return guarded(h, [&] {
        FEDD_CUDA(cudaSetDevice(h->device));
        if (count == 0) return;
        DBuf<double> dd;
        DBuf<float> db;
        dd.alloc(count);
        db.alloc((size_t)count * 9);
        k_element_geometry<<<ceil_div(count, 128), 128>>>(h->xyz.p, h->conn.p, h->ne, first, count, dd.p, db.p);
        FEDD_CUDA(cudaGetLastError());
        FEDD_CUDA(cudaMemcpy(det, dd.p, count * sizeof(double), cudaMemcpyDeviceToHost));
        FEDD_CUDA(cudaMemcpy(binv, db.p, (size_t)count * 9 * sizeof(float), cudaMemcpyDeviceToHost));
    });
}

// FE::assemblyRHS with a source function (fedd_rhs_points / fedd_assemble_rhs).
extern "C" fedd_status fedd_rhs_points(fedd_assembler *h, double *xq, int32_t *nq) {
    if (!h || !nq) return FEDD_ERR_ARG;
    return guarded(h, [&] {
        const RhsRule R = make_rhs_rule(h->order);
        *nq = R.nq;
        if (!xq) return;
        FEDD_CUDA(cudaSetDevice(h->device));
        DBuf<double> d;
        d.alloc((size_t)h->ne * R.nq * 3);
        launch_rhs_points(h->xyz.p, h->conn.p, h->ne, R, d.p, 0);
        FEDD_CUDA(cudaMemcpy(xq, d.p, (size_t)h->ne * R.nq * 3 * sizeof(double), cudaMemcpyDeviceToHost));
    });
}

extern "C" fedd_status fedd_assemble_rhs(fedd_assembler *h, const double *fq, int32_t ncomp, double *rhs) {
    if (!h || !fq || !rhs || (ncomp != 1 && ncomp != 3)) return FEDD_ERR_ARG;
    return guarded(h, [&] {
        FEDD_CUDA(cudaSetDevice(h->device));
        const RhsRule R = make_rhs_rule(h->order);
        const size_t nf = (size_t)h->ne * R.nq * ncomp, nr = (size_t)h->nn * ncomp;
        DBuf<double> df, stage, dr;
        df.upload(fq, nf, 0);
        stage.alloc((size_t)h->ne * R.npe * ncomp);
        dr.alloc(nr);
        FEDD_CUDA(cudaMemset(h->d_err.p, 0, sizeof(int)));
        launch_rhs_assemble(h->g, h->xyz.p, h->conn.p, h->ne, R, df.p, ncomp, stage.p, dr.p, h->d_err.p, 0);
        read_dev_error(h, 0);
        FEDD_CUDA(cudaMemcpy(rhs, dr.p, nr * sizeof(double), cudaMemcpyDeviceToHost));
    });
}
