"""C++ facade (include/mpflow_gb300.hpp): compiles against the library on the
CPU; on the GPU a differential reconstruction through mpFlow's class names
agrees with the Python binding of the same C ABI."""
import json
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "facade_demo.cpp")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def _build(tmp_path):
    import mpflow_gb300  # noqa: F401  (library built by the session fixture)
    libdir = os.path.join(ROOT, "mpflow_gb300", "_lib")
    exe = str(tmp_path / "facade_demo")
    cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), "-I", os.path.join(CUDA, "include"),
           SRC, "-o", exe, "-L", libdir, "-lmpflow_gb300", f"-Wl,-rpath,{libdir}",
           "-L", os.path.join(CUDA, "lib64"), "-lcudart", f"-Wl,-rpath,{os.path.join(CUDA, 'lib64')}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_facade_compiles_and_links(tmp_path):
    assert os.path.exists(_build(tmp_path))


def test_facade_json_reader(tmp_path):
    r = subprocess.run([_build(tmp_path), "json-selftest"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and json.loads(r.stdout)["json_selftest"], (r.stdout, r.stderr)


@pytest.mark.gpu
def test_solver_from_config_matches_python(tmp_path):
    """Solver::fromConfig on a mesh directory + JSON config (the reference's
    on-disk format) reconstructs what the Python binding computes."""
    import torch
    import mpflow_gb300 as mp
    from conftest import inclusion_sigma, make_setup
    exe = _build(tmp_path)
    mesh, src, _ = make_setup(rings=16, ports=16)
    d = tmp_path / "case"
    (d / "mesh").mkdir(parents=True)
    np.savetxt(d / "mesh" / "nodes.txt", mesh.nodes, fmt="%.17g")
    np.savetxt(d / "mesh" / "elements.txt", mesh.elements, fmt="%d")
    pat = mp.adjacent_pattern(16).astype(int).tolist()
    model = mp.EIT(mesh, src, 1.0)
    E = mesh.elements.shape[0]
    opts = mp.SolveOptions(tol=1e-6)
    V0, J = model.solve(torch.ones((1, E), device="cuda"), opts, jacobian=True)
    Vm = model.solve(torch.tensor(inclusion_sigma(mesh, seed=3), dtype=torch.float32, device="cuda")[None], opts)
    np.savetxt(d / "measurement.txt", Vm[0].cpu().numpy(), fmt="%.9g")
    factor = float(np.sqrt(0.1 * (J[0].cpu().numpy().astype(np.float64) ** 2).sum(axis=0).mean()))
    cfg = {"model": {"mesh": "mesh", "ports": {"count": 16, "width": 0.1, "offset": 0.0},
                     "source": {"type": "current", "value": 1e-3, "drivePattern": pat, "measurementPattern": pat},
                     "material": 1.0},
           "solver": {"parallelImages": 1, "regularizationFactor": factor, "regularizationType": "identity"}}
    (d / "config.json").write_text(json.dumps(cfg))
    r = subprocess.run([exe, "config", str(d)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, (r.stdout, r.stderr)
    got = np.loadtxt(d / "result.txt")
    Vmt = torch.tensor(np.loadtxt(d / "measurement.txt"), dtype=torch.float32, device="cuda")[None]
    want = 1.0 + model.inverse(J[0], V0, Vmt, factor, "identity")[0].cpu().numpy()
    # two independent forward solves at CG tolerance 1e-6 (the launch shapes
    # are autotuned by timing in each process, so the summation orders can
    # differ); the inverse amplifies their difference to ~3e-5 of the update
    assert np.abs(got - want).max() <= 1e-4 * max(np.abs(want - 1.0).max(), 1e-12) + 1e-6


@pytest.mark.gpu
def test_facade_reconstruction_matches_python(tmp_path):
    exe = _build(tmp_path)
    r = subprocess.run([exe, "16", "16"], capture_output=True, text=True, timeout=300)
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert r.returncode == 0 and out["ok"], (r.stdout, r.stderr)
    # the same forward solve through the Python binding
    import torch
    import mpflow_gb300 as mp
    from conftest import make_setup
    mesh, src, _ = make_setup(rings=16, ports=16)
    model = mp.EIT(mesh, src, 1.0)
    V = model.solve(torch.ones((1, mesh.elements.shape[0]), device="cuda"), mp.SolveOptions(tol=1e-7))
    V = V[0].cpu().numpy().astype(np.float64)
    assert abs(V.sum() - out["sum_v"]) <= 1e-6 * np.abs(V).sum()
    assert abs(np.abs(V).sum() - out["sum_abs_v"]) <= 1e-6 * np.abs(V).sum()


@pytest.mark.gpu
def test_facade_complex_reconstruction_matches_python(tmp_path):
    """models::EIT / solver::Solver instantiated on a complex data type (the
    reference's thrust::complex<float> instantiations): forward solve and
    differential reconstruction through the facade agree with the Python
    binding of mpf_eit_forward_complex + mpf_inverse_solve_complex."""
    exe = _build(tmp_path)
    res_file = tmp_path / "complex_result.txt"
    r = subprocess.run([exe, "complex", "16", "16", str(res_file)], capture_output=True, text=True, timeout=300)
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert r.returncode == 0 and out["ok"], (r.stdout, r.stderr)
    got = np.loadtxt(res_file)
    got = got[:, 0] + 1j * got[:, 1]
    import torch
    import mpflow_gb300 as mp
    from conftest import make_setup
    mesh, src, _ = make_setup(rings=16, ports=16)
    model = mp.EIT(mesh, src, 1.0)
    E = mesh.elements.shape[0]
    opts = mp.SolveOptions(tol=1e-7, solver="bicgstab")
    ref = torch.full((1, E), 1.0 + 0.15j, dtype=torch.complex64, device="cuda")
    V0, J = model.solve_complex(ref, opts, jacobian=True)
    c = mesh.nodes[mesh.elements].mean(axis=1)
    inside = (c[:, 0] - 0.3) ** 2 + (c[:, 1] - 0.2) ** 2 < 0.0625
    g = ref.clone()
    g[0, torch.tensor(inside, device="cuda")] = 0.5 + 0.3j
    Vt = model.solve_complex(g, opts)
    V0n = V0[0].cpu().numpy()
    scale = np.abs(V0n).sum()
    assert abs(V0n.real.sum() - out["sum_v_re"]) <= 1e-5 * scale
    assert abs(V0n.imag.sum() - out["sum_v_im"]) <= 1e-5 * scale
    want = (1.0 + 0.15j) + model.inverse_complex(J[0], V0, Vt, out["factor"], "identity")[0].cpu().numpy()
    delta = np.abs(want - (1.0 + 0.15j)).max()
    assert delta > 1e-3
    assert np.abs(got - want).max() <= 1e-4 * delta


def test_facade_instantiates_on_thrust_complex(tmp_path):
    """The reference's instantiations compile against the facade with its own
    data types: thrust::complex<float>, double and thrust::complex<double>
    (solver::Solver, solver::Inverse and models::EIT explicitly instantiated,
    every member); complex detection checked at compile time."""
    cccl = os.path.join(CUDA, "include", "cccl")
    if not os.path.exists(os.path.join(cccl, "thrust", "complex.h")):
        pytest.skip("thrust headers not found")
    src = tmp_path / "thrust_complex.cpp"
    src.write_text(
        "#include <thrust/complex.h>\n"
        "#include \"mpflow_gb300.hpp\"\n"
        "using namespace mpFlow;\n"
        "typedef thrust::complex<float> tc;\n"
        "typedef models::EIT<numeric::ConjugateGradient, FEM::Equation<tc, FEM::basis::Linear, false>> M1;\n"
        "typedef models::EIT<numeric::BiCGSTAB, FEM::Equation<tc, FEM::basis::Linear, true>> M2;\n"
        "template class models::EIT<numeric::ConjugateGradient, FEM::Equation<tc, FEM::basis::Linear, false>>;\n"
        "template class solver::Inverse<tc, numeric::ConjugateGradient>;\n"
        "template class solver::Solver<M1>;\n"
        "template class solver::Solver<M2, numeric::BiCGSTAB>;\n"
        "typedef models::EIT<numeric::ConjugateGradient, FEM::Equation<double, FEM::basis::Linear, false>> M3;\n"
        "typedef thrust::complex<double> td;\n"
        "typedef models::EIT<numeric::BiCGSTAB, FEM::Equation<td, FEM::basis::Linear, true>> M4;\n"
        "template class solver::Solver<M3>;\n"
        "template class solver::Solver<M4, numeric::BiCGSTAB>;\n"
        "template class solver::Inverse<double, numeric::ConjugateGradient>;\n"
        "static_assert(!detail::lib_native<double>() && !detail::lib_native<td>(), \"converted through FP32\");\n"
        "static_assert(detail::is_complex<tc>::value, \"thrust::complex is complex\");\n"
        "static_assert(!detail::is_complex<float>::value, \"float is real\");\n"
        "static_assert(sizeof(tc) == 2 * sizeof(float), \"interleaved pair\");\n")
    cmd = ["g++", "-std=c++17", "-fsyntax-only", "-I", os.path.join(ROOT, "include"), "-I",
           os.path.join(CUDA, "include"), "-I", cccl, str(src)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_facade_precision_conversion(tmp_path):
    """Wider data types (double, complex<double>) go through the library's
    FP32 interface by value conversion (detail::convert_value), checked
    here without a GPU."""
    cccl = os.path.join(CUDA, "include", "cccl")
    if not os.path.exists(os.path.join(cccl, "thrust", "complex.h")):
        pytest.skip("thrust headers not found")
    src = tmp_path / "convert.cpp"
    src.write_text(
        "#include <thrust/complex.h>\n#include <cstdio>\n#include \"mpflow_gb300.hpp\"\nusing namespace mpFlow;\n"
        "int main() {\n"
        "  bool ok = detail::convert_value<double>(1.5f) == 1.5 && detail::convert_value<float>(2.0) == 2.0f;\n"
        "  auto z = detail::convert_value<std::complex<float>>(thrust::complex<double>(1.25, -2.5));\n"
        "  auto w = detail::convert_value<thrust::complex<double>>(std::complex<float>(0.5f, 3.f));\n"
        "  ok = ok && z.real() == 1.25f && z.imag() == -2.5f && w.real() == 0.5 && w.imag() == 3.0;\n"
        "  std::printf(ok ? \"ok\\n\" : \"fail\\n\");\n  return ok ? 0 : 1;\n}\n")
    exe = str(tmp_path / "convert")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), "-I",
                        os.path.join(CUDA, "include"), "-I", cccl, str(src), "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and r.stdout.strip() == "ok", (r.stdout, r.stderr)


@pytest.mark.gpu
def test_facade_double_and_complex_double_match_float(tmp_path):
    """models::EIT and solver::Solver instantiated on double and
    complex<double> (the reference instantiates both natively,
    src/models/eit.cpp:273-304) against float and complex<float> on the same
    mesh and inputs: voltages (padded result layout), Jacobian (dataRows x
    E), fields after updateFields (two 2.5D components, complex for the
    complex types) and a solveDifferential reconstruction agree within 1e-5
    relative."""
    exe = _build(tmp_path)
    r = subprocess.run([exe, "wide", "16", "16"], capture_output=True, text=True, timeout=300)
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert r.returncode == 0 and out["ok"], (r.stdout, r.stderr)
    for k in ("double_v", "double_j", "double_fields", "double_sigma", "cdouble_v", "cdouble_j", "cdouble_sigma",
              "cdouble_fields"):
        assert out[k] <= 1e-5, (k, out)
    assert out["fields_values"] > 0 and out["sigma_min"] < 1.0
