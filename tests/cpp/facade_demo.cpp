// Reconstruction through the C++ facade with mpFlow's class names: a forward
// solve, a differential reconstruction of a low-conductivity inclusion, and a
// text round trip of the voltages.  Prints one JSON line; exit status 0 when
// every check holds.  Usage: facade_demo <rings> <electrodes>
//        facade_demo complex <rings> <electrodes> <result file>: the complex
//        (thrust::complex-style) model and differential reconstruction
//        facade_demo wide <rings> <electrodes>: double and complex<double>
//        instantiations against float and complex<float>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <sstream>
#include <string>

#include "mpflow_gb300.hpp"

using namespace mpFlow;
typedef models::EIT<numeric::ConjugateGradient, FEM::Equation<float, FEM::basis::Linear, false>> Model;
typedef models::EIT<numeric::BiCGSTAB, FEM::Equation<float, FEM::basis::Linear, false>> ModelBi;
typedef std::complex<float> cfloat;
typedef models::EIT<numeric::ConjugateGradient, FEM::Equation<cfloat, FEM::basis::Linear, false>> ModelZ;

// complex admittivity: forward solve at 1 + 0.15i, an inclusion of
// 0.5 + 0.3i at (0.3, 0.2) radius 0.25, solveDifferential with the identity
// regulariser; writes the reconstruction (re im per element) to `file`
static int complex_case(unsigned rings, unsigned L, std::string const& file) {
    cudaStream_t stream = nullptr;
    cublasHandle_t handle = nullptr;
    auto mesh = numeric::IrregularMesh::ring(rings);
    auto ports = FEM::Ports::circularBoundary(L, 0.1, mesh);
    auto pattern = std::make_shared<numeric::Matrix<int>>(L, L, stream);
    for (unsigned j = 0; j < L; ++j) {
        (*pattern)(j, j) = 1;
        (*pattern)((j + 1) % L, j) = -1;
    }
    pattern->copyToDevice(stream);
    auto sources = std::make_shared<FEM::Sources<cfloat>>(FEM::Sources<cfloat>::Open, cfloat(1e-3f), ports, pattern,
                                                          pattern, stream);
    auto model = std::make_shared<ModelZ>(mesh, sources, cfloat(1.f), handle, stream, 1, 1.0, 1.0);
    model->options.tol = 1e-7;
    const unsigned E = mesh->elements.rows();
    auto target = std::make_shared<numeric::Matrix<cfloat>>(E, 1, stream, cfloat(1.f, 0.15f));
    for (unsigned e = 0; e < E; ++e) {
        auto xy = mesh->elementNodes(e);
        const double cx = (xy(0, 0) + xy(1, 0) + xy(2, 0)) / 3.0, cy = (xy(0, 1) + xy(1, 1) + xy(2, 1)) / 3.0;
        if ((cx - 0.3) * (cx - 0.3) + (cy - 0.2) * (cy - 0.2) < 0.0625) (*target)(e, 0) = cfloat(0.5f, 0.3f);
    }
    target->copyToDevice(stream);
    solver::Solver<ModelZ> solver(model, 1, handle, stream);
    solver.referenceDistribution->fill(cfloat(1.f, 0.15f), stream);
    solver.preSolve(handle, stream);
    auto V0 = solver.calculation[0];
    V0->copyToHost(stream);
    double sumRe = 0.0, sumIm = 0.0;
    for (unsigned i = 0; i < V0->rows; ++i)
        for (unsigned j = 0; j < V0->cols; ++j) {
            sumRe += (*V0)(i, j).real();
            sumIm += (*V0)(i, j).imag();
        }
    auto Vt = model->solve(target, handle, stream);
    solver.measurement[0]->copy(Vt, stream);
    solver.inverseSolver->updateJacobian(model->jacobian, handle, stream);
    // the Jacobian of the reference distribution (preSolve's), for the factor
    model->solve(solver.referenceDistribution, handle, stream);
    const size_t nj = (size_t)model->jacobian->dataRows * E;
    std::vector<cfloat> J(nj);
    cudaMemcpy(J.data(), model->jacobian->deviceData, sizeof(cfloat) * nj, cudaMemcpyDeviceToHost);
    double jj = 0.0;
    for (auto v : J) jj += std::norm(v);
    const float factor = (float)(0.05 * std::sqrt(jj / model->jacobian->rows));
    solver.inverseSolver->setRegularizationParameter(cfloat(factor), solver::Inverse<cfloat>::identity, handle, stream);
    auto sigma = solver.solveDifferential(handle, stream);
    std::vector<cfloat> s(E);
    cudaMemcpy(s.data(), sigma->deviceData, sizeof(cfloat) * E, cudaMemcpyDeviceToHost);
    FILE* f = fopen(file.c_str(), "w");
    if (!f) return 3;
    for (auto v : s) fprintf(f, "%.9g %.9g\n", v.real(), v.imag());
    fclose(f);
    printf("{\"complex\": true, \"sum_v_re\": %.9e, \"sum_v_im\": %.9e, \"factor\": %.9e, \"ok\": true}\n", sumRe,
           sumIm, factor);
    return 0;
}

// The double and complex<double> instantiations against float and
// complex<float> on the same inputs: forward voltages, Jacobian, fields (real
// only) and a differential reconstruction through solver::Solver.  Prints the
// largest relative difference of each.
template <class T>
static std::vector<T> device_values(T const* p, size_t n) {
    std::vector<T> h(n);
    cudaMemcpy(h.data(), p, sizeof(T) * n, cudaMemcpyDeviceToHost);
    return h;
}
template <class A, class B>
static double rel_diff(std::vector<A> const& a, std::vector<B> const& b) {
    double d = 0.0, m = 0.0;
    for (size_t i = 0; i < a.size(); ++i) {
        const std::complex<double> x(detail::real_part(a[i]), detail::imag_part(a[i]));
        const std::complex<double> y(detail::real_part(b[i]), detail::imag_part(b[i]));
        d = std::max(d, std::abs(x - y));
        m = std::max(m, std::abs(y));
    }
    return d / std::max(m, 1e-300);
}

template <class T>
static std::shared_ptr<solver::Solver<models::EIT<numeric::ConjugateGradient, FEM::Equation<T, FEM::basis::Linear, false>>>>
wide_case(unsigned rings, unsigned L, T inclusion, T background, std::vector<T>* V, std::vector<T>* J,
          std::vector<T>* F, std::vector<T>* S) {
    typedef models::EIT<numeric::ConjugateGradient, FEM::Equation<T, FEM::basis::Linear, false>> M;
    cudaStream_t stream = nullptr;
    cublasHandle_t handle = nullptr;
    auto mesh = numeric::IrregularMesh::ring(rings);
    auto ports = FEM::Ports::circularBoundary(L, 0.1, mesh);
    auto pattern = std::make_shared<numeric::Matrix<int>>(L, L, stream);
    for (unsigned j = 0; j < L; ++j) {
        (*pattern)(j, j) = 1;
        (*pattern)((j + 1) % L, j) = -1;
    }
    pattern->copyToDevice(stream);
    auto sources = std::make_shared<FEM::Sources<T>>(FEM::Sources<T>::Open, T(1e-3), ports, pattern, pattern, stream);
    auto model = std::make_shared<M>(mesh, sources, T(1), handle, stream, 2, 1.0, 1.0);
    model->options.tol = 1e-7;
    const unsigned E = mesh->elements.rows();
    auto target = std::make_shared<numeric::Matrix<T>>(E, 1, stream, background);
    for (unsigned e = 0; e < E; ++e) {
        auto xy = mesh->elementNodes(e);
        const double cx = (xy(0, 0) + xy(1, 0) + xy(2, 0)) / 3.0, cy = (xy(0, 1) + xy(1, 1) + xy(2, 1)) / 3.0;
        if ((cx - 0.3) * (cx - 0.3) + (cy - 0.2) * (cy - 0.2) < 0.0625) (*target)(e, 0) = inclusion;
    }
    target->copyToDevice(stream);
    auto solver = std::make_shared<solver::Solver<M>>(model, 1, handle, stream);
    solver->referenceDistribution->fill(background, stream);
    solver->preSolve(handle, stream);
    auto V0 = solver->calculation[0];
    *V = device_values(V0->deviceData, (size_t)V0->dataRows * V0->cols);
    *J = device_values(model->jacobian->deviceData, (size_t)model->jacobian->dataRows * E);
    model->updateFields(stream);
    F->clear();
    for (auto const& f : model->fields) {
        auto h = device_values(f->deviceData, (size_t)f->dataRows * f->cols);
        F->insert(F->end(), h.begin(), h.end());
    }
    auto Vt = model->solve(target, handle, stream);
    solver->measurement[0]->copy(Vt, stream);
    model->solve(solver->referenceDistribution, handle, stream);
    solver->inverseSolver->updateJacobian(model->jacobian, handle, stream);
    solver->inverseSolver->setRegularizationParameter(T(2e-4), solver::Inverse<T>::identity, handle, stream);
    auto sigma = solver->solveDifferential(handle, stream);
    *S = device_values(sigma->deviceData, E);
    return solver;
}

static int wide(unsigned rings, unsigned L) {
    std::vector<float> Vf, Jf, Ff, Sf;
    std::vector<double> Vd, Jd, Fd, Sd;
    wide_case<float>(rings, L, 0.5f, 1.0f, &Vf, &Jf, &Ff, &Sf);
    wide_case<double>(rings, L, 0.5, 1.0, &Vd, &Jd, &Fd, &Sd);
    typedef std::complex<double> cdouble;
    std::vector<cfloat> Vz, Jz, Fz, Sz;
    std::vector<cdouble> Vw, Jw, Fw, Sw;
    wide_case<cfloat>(rings, L, cfloat(0.5f, 0.3f), cfloat(1.f, 0.15f), &Vz, &Jz, &Fz, &Sz);
    wide_case<cdouble>(rings, L, cdouble(0.5, 0.3), cdouble(1.0, 0.15), &Vw, &Jw, &Fw, &Sw);
    const double dv = rel_diff(Vd, Vf), dj = rel_diff(Jd, Jf), df = rel_diff(Fd, Ff), ds = rel_diff(Sd, Sf);
    const double zv = rel_diff(Vw, Vz), zj = rel_diff(Jw, Jz), zs = rel_diff(Sw, Sz), zf = rel_diff(Fw, Fz);
    double sMin = 1e300;
    for (double v : Sd) sMin = std::min(sMin, v);
    const bool sizes = Vd.size() == Vf.size() && Jd.size() == Jf.size() && Fd.size() == Ff.size() && !Fd.empty() &&
                       Sd.size() == Sf.size() && Vw.size() == Vz.size() && Jw.size() == Jz.size() &&
                       Sw.size() == Sz.size() && Fw.size() == Fz.size() && !Fz.empty();
    const bool ok = sizes && dv <= 1e-5 && dj <= 1e-5 && df <= 1e-5 && ds <= 1e-5 && zv <= 1e-5 && zj <= 1e-5 &&
                    zs <= 1e-5 && zf <= 1e-5 && sMin < 1.0;
    printf("{\"double_v\": %.3e, \"double_j\": %.3e, \"double_fields\": %.3e, \"double_sigma\": %.3e, "
           "\"cdouble_v\": %.3e, \"cdouble_j\": %.3e, \"cdouble_sigma\": %.3e, \"cdouble_fields\": %.3e, "
           "\"fields_values\": %zu, "
           "\"sigma_min\": %.6f, \"ok\": %s}\n",
           dv, dj, df, ds, zv, zj, zs, zf, Fd.size(), sMin, ok ? "true" : "false");
    return ok ? 0 : 1;
}

// json-selftest: parse a configuration without touching the GPU
static int json_selftest() {
    auto v = json::parse(R"({"model": {"mesh": {"rings": 12, "radius": 1.5}, "ports": {"count": 8, "width": 0.2,
        "clockwise": true}, "source": {"type": "voltage", "value": [1, 2.5e-3], "drivePattern": [[1, 0], [-1, 1]]},
        "2.5D": {"components": 3, "height": 2.0}, "material": {"referenceValue": 0.5}},
        "solver": {"regularizationType": "noser", "parallelImages": 2, "note": "a \"quoted\" word"}})");
    const bool ok = v["model"]["mesh"]["rings"].asInt() == 12 && v["model"]["mesh"]["radius"].asDouble() == 1.5 &&
                    v["model"]["ports"]["clockwise"].asBool() && v["model"]["source"]["value"][1].asDouble() == 2.5e-3 &&
                    v["model"]["source"]["drivePattern"][1][0].asInt() == -1 &&
                    v["model"]["2.5D"]["components"].asInt() == 3 && v["solver"]["regularizationType"].asString() == "noser" &&
                    v["solver"]["note"].asString() == "a \"quoted\" word" && v["solver"]["missing"].type == json::value::none &&
                    v["model"]["material"]["referenceValue"].asDouble() == 0.5;
    printf("{\"json_selftest\": %s}\n", ok ? "true" : "false");
    return ok ? 0 : 1;
}

// config <dir>: Solver::fromConfig(<dir>/config.json), measurement from
// <dir>/measurement.txt, differential reconstruction into <dir>/result.txt
static int from_config(std::string const& dir) {
    cudaStream_t stream = nullptr;
    cublasHandle_t handle = nullptr;
    auto config = json::parse_file(dir + "/config.json");
    auto solver = solver::Solver<Model>::fromConfig(config, handle, stream, dir);
    auto meas = numeric::Matrix<float>::loadtxt(dir + "/measurement.txt", stream);
    solver->measurement[0]->copy(meas, stream);
    auto sigma = solver->solveDifferential(handle, stream);
    const unsigned E = solver->forwardModel->mesh->elements.rows();
    numeric::Matrix<float> out(E, 1, stream);
    std::vector<float> s(E);
    cudaMemcpy(s.data(), sigma->deviceData, sizeof(float) * E, cudaMemcpyDeviceToHost);
    for (unsigned e = 0; e < E; ++e) out(e, 0) = s[e];
    out.savetxt(dir + "/result.txt");
    printf("{\"elements\": %u, \"ok\": true}\n", E);
    return 0;
}

int main(int argc, char** argv) {
    if (argc > 1 && std::string(argv[1]) == "json-selftest") return json_selftest();
    if (argc > 4 && std::string(argv[1]) == "complex") {
        try {
            return complex_case((unsigned)atoi(argv[2]), (unsigned)atoi(argv[3]), argv[4]);
        } catch (std::exception const& ex) {
            printf("{\"error\": \"%s\", \"ok\": false}\n", ex.what());
            return 2;
        }
    }
    if (argc > 3 && std::string(argv[1]) == "wide") {
        try {
            return wide((unsigned)atoi(argv[2]), (unsigned)atoi(argv[3]));
        } catch (std::exception const& ex) {
            printf("{\"error\": \"%s\", \"ok\": false}\n", ex.what());
            return 2;
        }
    }
    if (argc > 2 && std::string(argv[1]) == "config") {
        try {
            return from_config(argv[2]);
        } catch (std::exception const& ex) {
            printf("{\"error\": \"%s\", \"ok\": false}\n", ex.what());
            return 2;
        }
    }
    const unsigned rings = argc > 1 ? (unsigned)atoi(argv[1]) : 16;
    const unsigned L = argc > 2 ? (unsigned)atoi(argv[2]) : 16;
    cudaStream_t stream = nullptr;
    cublasHandle_t handle = nullptr;
    try {
        auto mesh = numeric::IrregularMesh::ring(rings);
        auto ports = FEM::Ports::circularBoundary(L, 0.1, mesh);
        auto pattern = std::make_shared<numeric::Matrix<int>>(L, L, stream);
        for (unsigned j = 0; j < L; ++j) {
            (*pattern)(j, j) = 1;
            (*pattern)((j + 1) % L, j) = -1;
        }
        pattern->copyToDevice(stream);
        auto sources = std::make_shared<FEM::Sources<float>>(FEM::Sources<float>::Open, 1e-3f, ports, pattern, pattern,
                                                            stream);
        auto model = std::make_shared<Model>(mesh, sources, 1.0f, handle, stream, 1, 1.0, 1.0);
        model->options.tol = 1e-7;
        const unsigned E = mesh->elements.rows();

        // forward solve at the reference conductivity
        auto reference = std::make_shared<numeric::Matrix<float>>(E, 1, stream, 1.0f);
        unsigned steps = 0;
        auto V0 = model->solve(reference, handle, stream, &steps);
        V0->copyToHost(stream);
        double sumV = 0.0, sumAbs = 0.0;
        for (unsigned i = 0; i < V0->rows; ++i)
            for (unsigned j = 0; j < V0->cols; ++j) {
                sumV += (*V0)(i, j);
                sumAbs += std::fabs((*V0)(i, j));
            }

        // the same solve with the BiCGSTAB solver tag
        auto modelBi = std::make_shared<ModelBi>(mesh, sources, 1.0f, handle, stream, 1, 1.0, 1.0);
        modelBi->options.tol = 1e-7;
        unsigned stepsBi = 0;
        auto Vb = modelBi->solve(reference, handle, stream, &stepsBi);
        Vb->copyToHost(stream);
        double biErr = 0.0, vMax = 0.0;
        for (unsigned i = 0; i < V0->rows; ++i)
            for (unsigned j = 0; j < V0->cols; ++j) {
                biErr = std::max(biErr, (double)std::fabs((*Vb)(i, j) - (*V0)(i, j)));
                vMax = std::max(vMax, (double)std::fabs((*V0)(i, j)));
            }
        biErr /= std::max(vMax, 1e-300);

        // standalone sparse matrix and solvers: a diagonally dominant 1-D
        // Laplacian from a dense matrix, x = A^-1 b by CG and BiCGSTAB
        const unsigned ns = 200, nrhs = 3;
        auto dense = std::make_shared<numeric::Matrix<float>>(ns, ns, stream);
        for (unsigned i = 0; i < ns; ++i) {
            (*dense)(i, i) = 3.f;
            if (i > 0) (*dense)(i, i - 1) = -1.f;
            if (i + 1 < ns) (*dense)(i, i + 1) = -1.f;
        }
        dense->copyToDevice(stream);
        auto As = std::make_shared<numeric::SparseMatrix<float>>(dense, stream);
        auto KInv = std::make_shared<numeric::SparseMatrix<float>>(ns, ns, stream);
        numeric::preconditioner::diagonal<float>(std::shared_ptr<numeric::SparseMatrix<float> const>(As), stream, KInv);
        const bool precondOk = KInv->density == 1 && std::fabs(KInv->getValue(5, 5) - 1.f / 3.f) < 1e-7f;
        auto bs = std::make_shared<numeric::Matrix<float>>(ns, nrhs, stream);
        for (unsigned j = 0; j < nrhs; ++j)
            for (unsigned i = 0; i < ns; ++i) (*bs)(i, j) = (float)std::sin(0.1 * (i + 1) * (j + 1));
        bs->copyToDevice(stream);
        double sparseErr = 0.0;
        unsigned cgSteps = 0, biSteps = 0;
        for (int which = 0; which < 2; ++which) {
            auto xs = std::make_shared<numeric::Matrix<float>>(ns, nrhs, stream);
            if (which == 0) {
                numeric::ConjugateGradient<float> cg(ns, nrhs, stream);
                cgSteps = cg.solve<numeric::SparseMatrix>(As, bs, handle, stream, xs, KInv);
            } else {
                numeric::BiCGSTAB<float> bi(ns, nrhs, stream);
                biSteps = bi.solve<numeric::SparseMatrix>(As, bs, handle, stream, xs);
            }
            auto ys = std::make_shared<numeric::Matrix<float>>(ns, nrhs, stream);
            As->multiply(xs, stream, ys);
            ys->copyToHost(stream);
            for (unsigned j = 0; j < nrhs; ++j)
                for (unsigned i = 0; i < ns; ++i) sparseErr = std::max(sparseErr, (double)std::fabs((*ys)(i, j) - (*bs)(i, j)));
        }

        // measurement: an inclusion of 0.5 S/m at (0.3, 0.2), radius 0.25
        auto target = std::make_shared<numeric::Matrix<float>>(E, 1, stream, 1.0f);
        std::vector<int> inside;
        for (unsigned e = 0; e < E; ++e) {
            auto xy = mesh->elementNodes(e);
            const double cx = (xy(0, 0) + xy(1, 0) + xy(2, 0)) / 3.0, cy = (xy(0, 1) + xy(1, 1) + xy(2, 1)) / 3.0;
            if ((cx - 0.3) * (cx - 0.3) + (cy - 0.2) * (cy - 0.2) < 0.0625) {
                (*target)(e, 0) = 0.5f;
                inside.push_back((int)e);
            }
        }
        target->copyToDevice(stream);
        solver::Solver<Model> solver(model, 1, handle, stream);
        solver.preSolve(handle, stream);
        auto Vt = model->solve(target, handle, stream);
        solver.measurement[0]->copy(Vt, stream);
        // regularisation factor relative to the Jacobian's RMS row norm
        const size_t nj = (size_t)model->jacobian->dataRows * E;
        std::vector<float> J(nj);
        cudaMemcpy(J.data(), model->jacobian->deviceData, sizeof(float) * nj, cudaMemcpyDeviceToHost);
        double jj = 0.0;
        for (float v : J) jj += (double)v * v;
        const float factor = (float)(0.05 * std::sqrt(jj / model->jacobian->rows));
        solver.inverseSolver->setRegularizationParameter(factor, solver::Inverse<float>::identity, handle, stream);
        auto sigma = solver.solveDifferential(handle, stream);
        std::vector<float> s(E);
        cudaMemcpy(s.data(), sigma->deviceData, sizeof(float) * E, cudaMemcpyDeviceToHost);
        double in = 0.0, out = 0.0;
        std::vector<char> mark(E, 0);
        for (int e : inside) mark[e] = 1;
        for (unsigned e = 0; e < E; ++e) (mark[e] ? in : out) += s[e] - 1.0;
        in /= std::max<size_t>(inside.size(), 1);
        out /= std::max<size_t>(E - inside.size(), 1);

        // text round trip
        std::stringstream txt;
        V0->savetxt(txt);
        auto back = numeric::Matrix<float>::loadtxt(txt, stream);
        back->copyToHost(stream);
        double rt = 0.0;
        for (unsigned i = 0; i < V0->rows; ++i)
            for (unsigned j = 0; j < V0->cols; ++j) rt = std::max(rt, (double)std::fabs((*back)(i, j) - (*V0)(i, j)));

        const bool ok = steps > 0 && std::isfinite(sumAbs) && sumAbs > 0.0 && in < out && in < -0.01 &&
                        rt <= 1e-6 * sumAbs && stepsBi > 0 && biErr <= 1e-5 && cgSteps > 0 && biSteps > 0 &&
                        sparseErr <= 1e-5 && precondOk;
        printf("{\"steps\": %u, \"sum_v\": %.9e, \"sum_abs_v\": %.9e, \"mean_delta_inside\": %.6e, "
               "\"mean_delta_outside\": %.6e, \"text_roundtrip_max_err\": %.3e, \"bicgstab_steps\": %u, "
               "\"bicgstab_rel_err\": %.3e, \"sparse_cg_steps\": %u, \"sparse_bicgstab_steps\": %u, "
               "\"sparse_residual\": %.3e, \"ok\": %s}\n",
               steps, sumV, sumAbs, in, out, rt, stepsBi, biErr, cgSteps, biSteps, sparseErr, ok ? "true" : "false");
        return ok ? 0 : 1;
    } catch (std::exception const& ex) {
        printf("{\"error\": \"%s\", \"ok\": false}\n", ex.what());
        return 2;
    }
}
