// facade_main.cpp -- drives the C++ facade (include/feddgpu_fe.hpp) the way
// FEDDLib's fe_test_*.cpp drive FE::assembly*, and writes every result as a
// named raw array for tests/test_gpu_cpp_facade.py, which checks them against
// the FP64 oracle and the Python binding.
//
// Record format, repeated: char name[32] (zero padded), int32 type
// (0 = float64, 1 = int64, 2 = int32), int64 count, count values.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "feddgpu_fe.hpp"

namespace {

FILE *out = nullptr;

template <class T> void put(const char *name, int type, const std::vector<T> &v) {
    char n[32] = {0};
    std::strncpy(n, name, sizeof n - 1);
    const int64_t count = (int64_t)v.size();
    std::fwrite(n, 1, sizeof n, out);
    std::fwrite(&type, sizeof type, 1, out);
    std::fwrite(&count, sizeof count, 1, out);
    if (count) std::fwrite(v.data(), sizeof(T), (size_t)count, out);
}
void put(const char *name, const std::vector<double> &v) { put(name, 0, v); }
void put(const char *name, const std::vector<int64_t> &v) { put(name, 1, v); }
void put(const char *name, const std::vector<int32_t> &v) { put(name, 2, v); }
void put_csr(const std::string &prefix, const feddgpu::CsrMatrix &A) {
    put((prefix + "_rowptr").c_str(), A.rowptr);
    put((prefix + "_colind").c_str(), A.colind);
    put((prefix + "_values").c_str(), A.values);
}

std::vector<double> fourier(const feddgpu::Domain &d, uint64_t seed, int kmin, int kmax, double scale) {
    std::vector<double> u((size_t)d.numNodes() * 3);
    feddgpu::check(fedd_field_fourier(seed, kmin, kmax, d.numNodes(), d.coords.data(), scale, u.data()));
    return u;
}

}  // namespace

int main(int argc, char **argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: %s OUTPUT\n", argv[0]);
        return 2;
    }
    out = std::fopen(argv[1], "wb");
    if (!out) return 2;
    using namespace feddgpu;
    try {
        // ---- Navier-Stokes, as NavierStokesAssFE drives FE::assemblyNavierStokes
        Domain v = Domain::structured(2, "P2", 3), pr = Domain::structured(2, "P1", 3);
        std::vector<double> u = fourier(v, 3, 1, 4, 1.0);
        std::vector<double> p((size_t)pr.numNodes());
        check(fedd_field_uniform(3, pr.numNodes(), -1.0, 1.0, p.data()));
        ParameterList params;
        params.sublist("Parameter").set("Viscosity", 0.01).set("Density", 1.0);
        params.sublist("General").set("Linearization", "Newton");
        FE fe;
        fe.addFE(v);
        fe.addFE(pr);
        const std::array<std::array<double, 2>, 2> ones{{{1.0, 1.0}, {1.0, 1.0}}};
        BlockMatrix A;
        BlockMultiVector res;
        fe.assemblyNavierStokes(3, "P2", "P1", 2, 3, 1, u, p, A, res, ones, params, false, "Jacobian");
        put_csr("ns00", A.block[0][0]);
        put_csr("ns01", A.block[0][1]);
        put_csr("ns10", A.block[1][0]);
        put("ns11_nnz", std::vector<int64_t>{A.block[1][1].nnz()});
        fe.assemblyNavierStokes(3, "P2", "P1", 2, 3, 1, u, p, A, res, ones, params, false, "Rhs");
        put("ns_res_u", res.block[0]);
        put("ns_res_p", res.block[1]);
        // the residual's block factors (coeff, handed to the elements by setCoeff)
        const std::array<std::array<double, 2>, 2> co{{{0.5, 2.0}, {-1.5, 3.0}}};
        fe.assemblyNavierStokes(3, "P2", "P1", 2, 3, 1, u, p, A, res, co, params, false, "Rhs");
        put("ns_res_u_coeff", res.block[0]);
        put("ns_res_p_coeff", res.block[1]);
        BlockMatrix Afp;
        fe.assemblyNavierStokes(3, "P2", "P1", 2, 3, 1, u, p, Afp, res, ones, params, false, "FixedPoint");
        put("nsfp00_values", Afp.block[0][0].values);
        // reAssemble: block (0,0) only, in place
        fe.assemblyNavierStokes(3, "P2", "P1", 2, 3, 1, u, p, A, res, ones, params, true, "Jacobian");
        put("ns00_reassembled", A.block[0][0].values);

        // ---- generalized-Newtonian fluid, selected by Material/Newtonian = false,
        // with the outflow term on the faces of the plane x = 1
        {
            Domain gv = Domain::structured(2, "P2", 6), gp = Domain::structured(2, "P1", 6);
            static const int FV[4][3] = {{0, 1, 2}, {0, 1, 3}, {0, 2, 3}, {1, 2, 3}};
            for (int64_t e = 0; e < gv.numElements(); e++)
                for (const auto &f : FV) {
                    bool on = true;
                    for (int t = 0; t < 3; t++)
                        on = on && std::abs(gv.coords[(size_t)gv.elements[(size_t)e * 10 + f[t]] * 3] - 1.0) < 1e-12;
                    if (on)
                        for (int t = 0; t < 3; t++) gv.outflowFaces.push_back(gv.elements[(size_t)e * 10 + f[t]]);
                }
            put("gn_faces", gv.outflowFaces);
            std::vector<double> gu = fourier(gv, 6, 1, 4, 0.5);
            std::vector<double> gpv((size_t)gp.numNodes());
            check(fedd_field_uniform(6, gp.numNodes(), -1.0, 1.0, gpv.data()));
            ParameterList gpar;
            gpar.sublist("Parameter").set("Viscosity", 0.01).set("Density", 1.0);
            gpar.sublist("General").set("Linearization", "Newton");
            ParameterList &mat = gpar.sublist("Material");
            mat.set("Newtonian", false).set("ShearThinningModel", "Carreau-Yasuda");
            mat.set("CharacteristicTime_Lambda", 1.902).set("FluidIndex_n", 0.22);
            mat.set("ZeroShearRateViscosity_eta0", 0.056).set("InftyShearRateViscosity_etaInfty", 0.00345);
            mat.set("InflectionPoint_a", 1.25).set("Numerical_ZeroValue_ShearRate", 1e-12);
            FE gfe;
            gfe.addFE(gv);
            gfe.addFE(gp);
            BlockMatrix GA, GF;
            BlockMultiVector gres;
            gfe.assemblyNavierStokes(3, "P2", "P1", 2, 3, 1, gu, gpv, GA, gres, ones, gpar, false, "Jacobian");
            put_csr("gn00", GA.block[0][0]);
            gfe.assemblyNavierStokes(3, "P2", "P1", 2, 3, 1, gu, gpv, GA, gres, ones, gpar, false, "Rhs");
            put("gn_res_u", gres.block[0]);
            put("gn_res_p", gres.block[1]);
            gfe.assemblyNavierStokes(3, "P2", "P1", 2, 3, 1, gu, gpv, GF, gres, ones, gpar, false, "FixedPoint");
            put("gnfp00_values", GF.block[0][0].values);
            // the same element through the factory's "GeneralizedNewtonian" key
            AssembleFEFactory gfac;
            std::vector<double> gK, gr;
            std::vector<std::shared_ptr<AssembleFE>> gel;
            for (int e = 0; e < 4; e++) {
                std::vector<std::array<double, 3>> nodes(10);
                for (int a = 0; a < 10; a++)
                    for (int c = 0; c < 3; c++) nodes[a][c] = gv.coords[(size_t)gv.elements[(size_t)e * 10 + a] * 3 + c];
                gel.push_back(gfac.build("GeneralizedNewtonian", 0, nodes, gpar));
            }
            for (int e = 0; e < 4; e++) {
                std::vector<double> sol(34);
                for (int a = 0; a < 10; a++)
                    for (int d = 0; d < 3; d++) sol[3 * a + d] = gu[(size_t)gv.elements[(size_t)e * 10 + a] * 3 + d];
                for (int a = 0; a < 4; a++) sol[30 + a] = gpv[(size_t)gp.elements[(size_t)e * 4 + a]];
                gel[e]->updateSolution(sol);
            }
            for (int e = 0; e < 4; e++) {
                gel[e]->assembleJacobian();
                gel[e]->assembleRHS();
                auto K = gel[e]->getJacobian();
                auto r = gel[e]->getRHS();
                gK.insert(gK.end(), K.begin(), K.end());
                gr.insert(gr.end(), r.begin(), r.end());
            }
            put("assfe_gn_K", gK);
            put("assfe_gn_r", gr);
            std::vector<int32_t> gcode;
            try {
                gel[0]->assembleJacobianBlock(0);
                gcode.push_back(0);
            } catch (const Error &e) {
                gcode.push_back((int32_t)e.code);
            }
            put("assfe_gn_block_code", gcode);
        }

        // ---- AssembleFE elements through the factory (batched)
        AssembleFEFactory factory;
        std::vector<std::shared_ptr<AssembleFE>> elems;
        const int nel = 6;
        for (int e = 0; e < nel; e++) {
            std::vector<std::array<double, 3>> nodes(10);
            for (int a = 0; a < 10; a++)
                for (int c = 0; c < 3; c++) nodes[a][c] = v.coords[(size_t)v.elements[(size_t)e * 10 + a] * 3 + c];
            elems.push_back(factory.build("NavierStokes", 0, nodes, params));
        }
        std::vector<double> Kall, rall;
        for (int e = 0; e < nel; e++) {
            std::vector<double> sol(34);
            for (int a = 0; a < 10; a++)
                for (int d = 0; d < 3; d++) sol[3 * a + d] = u[(size_t)v.elements[(size_t)e * 10 + a] * 3 + d];
            for (int a = 0; a < 4; a++) sol[30 + a] = p[(size_t)pr.elements[(size_t)e * 4 + a]];
            elems[e]->updateSolution(sol);
        }
        for (int e = 0; e < nel; e++) {
            elems[e]->assembleJacobian();
            elems[e]->assembleRHS();
            auto K = elems[e]->getJacobian();
            auto r = elems[e]->getRHS();
            Kall.insert(Kall.end(), K.begin(), K.end());
            rall.insert(rall.end(), r.begin(), r.end());
        }
        put("assfe_ns_K", Kall);
        put("assfe_ns_r", rall);
        std::vector<int32_t> ctl_codes;
        {  // changeLinearization: FixedPoint from the parameter list, then Newton
            ParameterList fp;
            fp.sublist("Parameter").set("Viscosity", 0.01).set("Density", 1.0);
            fp.sublist("General").set("Linearization", "FixedPoint");
            AssembleFEFactory ffac;
            std::vector<std::shared_ptr<AssembleFE>> fel;
            for (int e = 0; e < nel; e++) {
                std::vector<std::array<double, 3>> nodes(10);
                for (int a = 0; a < 10; a++)
                    for (int c = 0; c < 3; c++) nodes[a][c] = v.coords[(size_t)v.elements[(size_t)e * 10 + a] * 3 + c];
                fel.push_back(ffac.build("NavierStokes", 0, nodes, fp));
                fel[e]->updateSolution(elems[e]->getSolution());
            }
            std::vector<double> Kfp, Knt;
            for (int e = 0; e < nel; e++) {
                fel[e]->assembleJacobian();
                fel[e]->assembleJacobianBlock(0);  // a no-op for this element type
                auto K = fel[e]->getJacobian();
                Kfp.insert(Kfp.end(), K.begin(), K.end());
            }
            for (int e = 0; e < nel; e++) fel[e]->changeLinearization("Newton");
            for (int e = 0; e < nel; e++) {
                fel[e]->assembleJacobian();
                auto K = fel[e]->getJacobian();
                Knt.insert(Knt.end(), K.begin(), K.end());
            }
            put("assfe_ns_fp_K", Kfp);
            put("assfe_ns_newton_K", Knt);
            const std::array<std::array<double, 2>, 2> co2{{{0.5, 2.0}, {-1.5, 3.0}}};
            std::vector<double> rco;
            for (int e = 0; e < nel; e++) fel[e]->setCoeff(co2);
            for (int e = 0; e < nel; e++) {
                fel[e]->assembleRHS();
                auto r = fel[e]->getRHS();
                rco.insert(rco.end(), r.begin(), r.end());
            }
            put("assfe_ns_coeff_r", rco);
            // one element on another linearization: the batch cannot be evaluated
            fel[2]->changeLinearization("FixedPoint");
            try {
                fel[0]->assembleJacobian();
                ctl_codes.push_back(0);
            } catch (const Error &e) {
                ctl_codes.push_back((int32_t)e.code);
            }
        }
        {  // updateParameter("E") on neo-Hooke elements, and the time / Newton counters
            Domain s2 = Domain::structured(2, "P2", 4);
            std::vector<double> d2 = fourier(s2, 4, 1, 2, 0.004);
            ParameterList ep2;
            ep2.sublist("Parameter").set("E", 32.0 / 11.0).set("Poisson Ratio", 5.0 / 11.0);
            AssembleFEFactory nfac;
            std::vector<std::shared_ptr<AssembleFE>> nel2;
            for (int e = 0; e < 4; e++) {
                std::vector<std::array<double, 3>> nodes(10);
                std::vector<double> sol(30);
                for (int a = 0; a < 10; a++) {
                    const int32_t g = s2.elements[(size_t)e * 10 + a];
                    for (int c = 0; c < 3; c++) {
                        nodes[a][c] = s2.coords[(size_t)g * 3 + c];
                        sol[3 * a + c] = d2[(size_t)g * 3 + c];
                    }
                }
                nel2.push_back(nfac.build("NonLinearElasticity", 0, nodes, ep2));
                nel2[e]->updateSolution(sol);
                nel2[e]->updateParameter("E", 5.0);
                nel2[e]->updateParameter("Poisson Ratio", 0.1);  // not a parameter the element updates
            }
            std::vector<double> K5, r5;
            for (int e = 0; e < 4; e++) {
                nel2[e]->assembleJacobian();
                nel2[e]->assembleRHS();
                auto K = nel2[e]->getJacobian();
                auto r = nel2[e]->getRHS();
                K5.insert(K5.end(), K.begin(), K.end());
                r5.insert(r5.end(), r.begin(), r.end());
            }
            put("assfe_nhE5_K", K5);
            put("assfe_nhE5_r", r5);
            nel2[3]->updateParameter("E", 7.0);
            try {
                nel2[0]->assembleJacobian();
                ctl_codes.push_back(0);
            } catch (const Error &e) {
                ctl_codes.push_back((int32_t)e.code);
            }
            nel2[0]->advanceInTime(0.5);
            nel2[0]->advanceInTime(0.25);
            nel2[0]->advanceNewtonStep();
            nel2[0]->advanceNewtonStep();
            put("assfe_counters", std::vector<double>{nel2[0]->getTimeStep(), nel2[0]->getTimeIncrement(),
                                                      (double)nel2[0]->getNewtonStep(), (double)nel2[1]->getNewtonStep()});
        }

        // ---- Laplace P1 + load, as Laplace_def.hpp drives FE::assemblyLaplace / assemblyRHS
        Domain l = Domain::structured(2, "P1", 1);
        FE fl;
        fl.addFE(l);
        CsrMatrix L;
        fl.assemblyLaplace(3, "P1", 1, L);
        put_csr("lap", L);
        BlockMatrix LA;  // the AssembleFE_Laplace route, as fe_test_laplace.cpp compares them
        fl.assemblyLaplaceAssFE(3, "P1", 1, 1, LA);
        put_csr("lapassfe", LA.block[0][0]);
        std::vector<double> b;
        fl.assemblyRHS(3, "P1", b, "Scalar", 1.0);
        put("lap_rhs", b);
        // a source function, FEDDLib's RhsFunc_Type: f(x, res, parameters)
        std::vector<double> bf, fpar{2.0};
        fl.assemblyRHS(3, "P1", bf, "Scalar",
                       [](double *x, double *r, double *par) { r[0] = par[0] * x[0] + std::sin(x[1]); }, fpar);
        put("lap_rhs_func", bf);

        // ---- nonlinear elasticity (skr2), tangent + residual
        Domain s = Domain::structured(2, "P2", 4);
        std::vector<double> d = fourier(s, 4, 1, 2, 0.004);
        ParameterList ep;
        ep.sublist("Parameter").set("E", 32.0 / 11.0).set("Poisson Ratio", 5.0 / 11.0);
        FE fs;
        fs.addFE(s);
        BlockMatrix K;
        BlockMultiVector r;
        fs.assemblyNonLinearElasticity(3, "P2", 2, 3, d, K, r, ep);
        put_csr("nh", K.block[0][0]);
        put("nh_res", r.block[0]);
        std::vector<double> bv, vpar{0.5};
        fs.assemblyRHS(
            3, "P2", bv, "Vector",
            [](double *x, double *r, double *par) {
                r[0] = x[0] * x[0];
                r[1] = par[0] * x[1];
                r[2] = 1.0 + x[2];
            },
            vpar);
        put("nh_rhs_vector", bv);
        {  // the E-field variant: a Young's modulus per element
            std::vector<double> emod((size_t)s.numElements());
            for (size_t e = 0; e < emod.size(); e++) emod[e] = 0.5 + 0.25 * (double)(e % 7);
            BlockMatrix KE;
            BlockMultiVector rE;
            fs.assemblyNonLinearElasticity(3, "P2", 2, 3, d, KE, rE, ep, s, emod);
            put("nhE_values", KE.block[0][0].values);
            put("nhE_rowptr", KE.block[0][0].rowptr);
            put("nhE_colind", KE.block[0][0].colind);
            put("nhE_res", rE.block[0]);
        }

        // ---- errors become exceptions with the engine's status code
        std::vector<int32_t> codes;
        try {
            CsrMatrix bad;
            fl.assemblyLaplace(3, "P3", 1, bad);
            codes.push_back(0);
        } catch (const Error &e) {
            codes.push_back((int32_t)e.code);
        }
        try {
            BlockMatrix bad;
            fe.assemblyNavierStokes(3, "P2", "P1", 2, 3, 1, std::vector<double>(5), p, bad, res, ones, params,
                                    false, "Jacobian");
            codes.push_back(0);
        } catch (const Error &e) {
            codes.push_back((int32_t)e.code);
        }
        put("error_codes", codes);
        put("assfe_ctl_codes", ctl_codes);
    } catch (const std::exception &e) {
        std::fprintf(stderr, "facade_main: %s\n", e.what());
        std::fclose(out);
        return 1;
    }
    std::fclose(out);
    return 0;
}
