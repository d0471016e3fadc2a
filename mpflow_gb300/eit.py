"""Host-side mirror of mpFlow's EIT interface over the C ABI.

Class and method names follow the reference (pgebhardt/mpflow):

* :class:`IrregularMesh`  -- numeric::IrregularMesh (include/mpflow/numeric/irregular_mesh.h:27-61)
* :class:`Ports`          -- FEM::Ports (include/mpflow/fem/ports.h:26-46)
* :class:`Sources`        -- FEM::Sources (include/mpflow/fem/sources.h:31-113)
* :class:`EIT`            -- models::EIT (include/mpflow/models/eit.h:31-81)

All numerics run in libmpflow_gb300.so on the GPU; this module only shapes
arguments.  Device buffers are torch CUDA tensors (used as plain device
memory); the stream is torch's current stream.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _ffi
from ._ffi import check, lib, ptr

OPEN, FIXED = 0, 1


def data_rows(n: int) -> int:
    """Padded row count of a reference dense matrix (src/numeric/matrix.cpp:49-55)."""
    return int(lib().mpf_data_rows(int(n)))


class IrregularMesh:
    """Triangle mesh with edge table and boundary (numeric::IrregularMesh)."""

    def __init__(self, nodes: np.ndarray, elements: np.ndarray):
        self.nodes = np.ascontiguousarray(nodes, dtype=np.float64)
        self.elements = np.ascontiguousarray(elements, dtype=np.int32)
        if self.nodes.ndim != 2 or self.nodes.shape[1] != 2:
            raise ValueError("mpFlow::numeric::IrregularMesh::IrregularMesh: nodes.cols() != 2")
        if self.elements.shape[0] == 0:
            raise ValueError("mpFlow::numeric::IrregularMesh::IrregularMesh: elements.rows() == 0")
        N, E = self.nodes.shape[0], self.elements.shape[0]
        edges = np.zeros((3 * E, 2), np.int32)
        element_edges = np.zeros((E, 3), np.int32)
        boundary = np.zeros(3 * E, np.int32)
        ne, nb = ctypes.c_int32(0), ctypes.c_int32(0)
        check(lib().mpf_mesh_edges(N, E, ptr(self.nodes), ptr(self.elements), ptr(edges),
                                   ptr(element_edges), ptr(boundary), ctypes.byref(ne),
                                   ctypes.byref(nb)))
        self.edges = edges[:ne.value].copy()
        self.elementEdges = element_edges
        self.boundary = boundary[:nb.value].copy()

    @staticmethod
    def ring(rings: int, radius: float = 1.0) -> "IrregularMesh":
        """Disk of `rings` concentric rings, ring i carrying 6i nodes."""
        n, e = ctypes.c_int32(0), ctypes.c_int32(0)
        check(lib().mpf_ring_mesh_counts(int(rings), ctypes.byref(n), ctypes.byref(e)))
        nodes = np.zeros((n.value, 2))
        elements = np.zeros((e.value, 3), np.int32)
        check(lib().mpf_ring_mesh(int(rings), float(radius), ptr(nodes), ptr(elements)))
        return IrregularMesh(nodes, elements)

    def elementNodes(self, element: int) -> np.ndarray:
        """Coordinates of the element's three nodes (IrregularMesh::elementNodes), 3 x 2."""
        return self.nodes[self.elements[element]]

    def edgeNodes(self, edge: int) -> np.ndarray:
        """Coordinates of the edge's two nodes (IrregularMesh::edgeNodes), 2 x 2."""
        return self.nodes[self.edges[edge]]


class Ports:
    """Electrode edge sets (FEM::Ports)."""

    def __init__(self, edges: np.ndarray):
        self.edges = np.ascontiguousarray(edges, dtype=np.int32)
        if self.edges.shape[0] == 0:
            raise ValueError("mpFlow::FEM::Ports::Ports: edges == 0")
        self.count = self.edges.shape[0]

    @staticmethod
    def circularBoundary(count: int, width: float, mesh: IrregularMesh, offset: float = 0.0,
                         clockwise: bool = False, cap: int = 512) -> "Ports":
        """`count` electrodes of `width` radians evenly spaced on the
        boundary from `offset` (FEM::Ports::circularBoundary,
        src/fem/ports.cpp:32-77, mpf_ports_circular); at most `cap` edges per
        port."""
        out = np.full((count, cap), -1, np.int32)
        mx = ctypes.c_int32(0)
        check(lib().mpf_ports_circular(mesh.nodes.shape[0], ptr(mesh.nodes), mesh.elements.shape[0],
                                       ptr(mesh.elements), ptr(mesh.edges), mesh.boundary.shape[0],
                                       ptr(mesh.boundary), int(count), float(width), float(offset),
                                       int(bool(clockwise)), ptr(out), cap, ctypes.byref(mx)))
        return Ports(out[:, :max(mx.value, 1)].copy())


def adjacent_pattern(count: int) -> np.ndarray:
    """Adjacent (+1 on port j, -1 on port j+1) pattern, ports x count."""
    p = np.zeros((count, count))
    for j in range(count):
        p[j, j] = 1.0
        p[(j + 1) % count, j] = -1.0
    return p


class Sources:
    """Excitation description (FEM::Sources): type, values and patterns."""

    Open, Fixed = OPEN, FIXED

    def __init__(self, type_: int, values, ports: Ports, drivePattern: np.ndarray,
                 measurementPattern: np.ndarray):
        if ports is None:
            raise ValueError("mpFlow::FEM::Sources::Sources: ports == nullptr")
        self.type = int(type_)
        self.ports = ports
        self.drivePattern = np.asfortranarray(drivePattern, dtype=np.float64)
        self.measurementPattern = np.asfortranarray(measurementPattern, dtype=np.float64)
        vals = np.atleast_1d(np.asarray(values, dtype=np.float64))
        if vals.size == 1:
            vals = np.full(self.drivePattern.shape[1], vals[0])
        if vals.size != self.drivePattern.shape[1]:
            raise ValueError("mpFlow::FEM::Sources::Sources: invalid size of values vector")
        self.values = vals

    @property
    def pattern(self) -> np.ndarray:
        """[values * drive | measurement] (src/fem/sources.cpp:58-71)."""
        return np.concatenate([self.drivePattern * self.values[None, :], self.measurementPattern], axis=1)


class SolveOptions:
    """mpf_solve_opts; preconditioner "jacobi" (the reference's) or
    "two-level" (Jacobi plus an aggregation coarse correction); solver "cg"
    (numeric::ConjugateGradient) or "bicgstab" (numeric::BiCGSTAB, Jacobi)."""

    PRECONDITIONERS = {"jacobi": 0, "two-level": 1}
    SOLVERS = {"cg": 0, "bicgstab": 1}
    # warm_start: False/0 cold, True/1/"previous" fields of the previous call,
    # 2/"homogeneous" fields of the homogeneous distribution
    WARM_STARTS = {False: 0, True: 1, 0: 0, 1: 1, 2: 2, "previous": 1, "homogeneous": 2}

    # gn_factor: factor of J J^T + mu I in the Gauss-Newton update
    GN_FACTORS = {"fp64": 0, "fp32-refined": 1}

    def __init__(self, tol=1e-6, max_iter=0, refine_tol=0.0, max_refine=6, warm_start=False,
                 check_every=16, preconditioner: str = "jacobi", solver: str = "cg",
                 gn_factor: str = "fp64", accept_tol: float = 0.0, accept_margin: float = 0.1):
        self.tol, self.max_iter, self.refine_tol = tol, max_iter, refine_tol
        self.max_refine, self.warm_start, self.check_every = max_refine, warm_start, check_every
        if warm_start not in self.WARM_STARTS:
            raise ValueError(f"warm_start must be one of {list(self.WARM_STARTS)}")
        if preconditioner not in self.PRECONDITIONERS:
            raise ValueError(f"preconditioner must be one of {sorted(self.PRECONDITIONERS)}")
        self.preconditioner = preconditioner
        if solver not in self.SOLVERS:
            raise ValueError(f"solver must be one of {sorted(self.SOLVERS)}")
        self.solver = solver
        if gn_factor not in self.GN_FACTORS:
            raise ValueError(f"gn_factor must be one of {sorted(self.GN_FACTORS)}")
        self.gn_factor = gn_factor
        # learned Gauss-Newton: tolerance of the acceptance solve and the
        # margin below the target that decides on it
        self.accept_tol, self.accept_margin = float(accept_tol), float(accept_margin)

    def c(self) -> _ffi.SolveOpts:
        """The options as the C ABI's mpf_solve_opts."""
        return _ffi.SolveOpts(float(self.tol), int(self.max_iter), float(self.refine_tol),
                              int(self.max_refine), self.WARM_STARTS[self.warm_start], int(self.check_every),
                              self.PRECONDITIONERS[self.preconditioner], self.SOLVERS[self.solver],
                              self.GN_FACTORS[self.gn_factor], self.accept_tol, self.accept_margin)


def _stream():
    import torch
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class EIT:
    """2.5D EIT forward model resident on one GPU (models::EIT).

    ``solve`` takes a (frames x elements) float32 CUDA tensor of material
    values and returns the (frames x meas x drive) electrode voltages."""

    def __init__(self, mesh: IrregularMesh, sources: Sources, referenceValue: float = 1.0,
                 components: int = 1, height: float = 1.0, portHeight: float = 1.0,
                 logarithmic: bool = False, device: int = 0, exact_jacobian: bool = False,
                 contact_impedance: float = 0.0):
        self.mesh, self.sources = mesh, sources
        self.contact_impedance = float(contact_impedance)
        self.referenceValue = float(referenceValue)
        self.components, self.height, self.portHeight = int(components), float(height), float(portHeight)
        self.logarithmic = bool(logarithmic)
        self.device = int(device)
        self._keep = [mesh.nodes, mesh.elements, mesh.edges, sources.ports.edges,
                      sources.drivePattern, sources.measurementPattern, sources.values]
        d = _ffi.EitDesc(
            mesh.nodes.shape[0], mesh.elements.shape[0], ptr(mesh.nodes).value, ptr(mesh.elements).value,
            ptr(mesh.edges).value, mesh.edges.shape[0], sources.ports.count,
            ptr(sources.ports.edges).value, sources.ports.edges.shape[1],
            sources.drivePattern.shape[1], sources.measurementPattern.shape[1],
            ptr(sources.drivePattern).value, ptr(sources.measurementPattern).value,
            ptr(sources.values).value, sources.type, self.referenceValue, int(self.logarithmic),
            self.components, self.height, self.portHeight, self.device, int(bool(exact_jacobian)),
            self.contact_impedance)
        h = ctypes.c_void_p()
        check(lib().mpf_eit_create(ctypes.byref(d), ctypes.byref(h)))
        self._h = h
        info = _ffi.EitInfo()
        check(lib().mpf_eit_get_info(h, ctypes.byref(info)))
        self.info = {name: getattr(info, name) for name, _ in _ffi.EitInfo._fields_}
        self.last_stats = None
        self.prior_lambda = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            lib().mpf_eit_destroy(h)
            self._h = None

    # -- shapes
    @property
    def jacobian_rows(self) -> int:
        """Rows of the Jacobian: drive count x measurement count, each padded to 16."""
        return self.info["jacobian_rows"]

    def _frames(self, gamma):
        import torch
        if not (isinstance(gamma, torch.Tensor) and gamma.is_cuda and gamma.dtype == torch.float32):
            raise TypeError("materialDistribution must be a float32 CUDA tensor")
        g = gamma.reshape(-1, self.mesh.elements.shape[0]).contiguous()
        return g, g.shape[0]

    def _vmeas(self, v_meas, F: int):
        """Measured voltages in the logical (frames, Mm, Md) shape that solve()
        returns -> the library's layout (column-major Mm x Md per frame)."""
        Mm, Md = self.info["meas_count"], self.info["drive_count"]
        return v_meas.reshape(F, Mm, Md).transpose(1, 2).contiguous()

    def assemble(self, gamma):
        """Stiffness and mass slot values in the reference ELL layout."""
        import torch
        g, F = self._frames(gamma)
        dr = self.info["data_rows"]
        S = torch.empty((F, dr, 32), dtype=torch.float32, device=g.device)
        R = torch.empty_like(S)
        check(lib().mpf_eit_assemble(self._h, F, ptr(g), ptr(S), ptr(R), _stream()))
        return S, R

    def solve(self, materialDistribution, options: SolveOptions | None = None, jacobian: bool = False,
              raise_on_noconv: bool = True):
        """Forward solve; returns V (frames x Mm x Md) and, if asked, J
        (frames x rowsJ x E, the reference's column-major jacobian as its
        transpose view).  With raise_on_noconv=False an iteration-cap hit is
        only recorded in last_stats.not_converged."""
        import torch
        g, F = self._frames(materialDistribution)
        Mm, Md = self.info["meas_count"], self.info["drive_count"]
        V = torch.empty((F, Md, Mm), dtype=torch.float32, device=g.device)
        J = None
        if jacobian:
            J = torch.empty((F, self.mesh.elements.shape[0], self.jacobian_rows), dtype=torch.float32,
                            device=g.device)
        st = _ffi.SolveStats()
        o = (options or SolveOptions()).c()
        status = lib().mpf_eit_forward(self._h, F, ptr(g), ptr(V), ptr(J), ctypes.byref(o), ctypes.byref(st),
                                       _stream())
        self.last_stats = st
        if status != _ffi.MPF_OK and (raise_on_noconv or status != 4):
            check(status)
        Vm = V.transpose(1, 2)  # (F, Mm, Md): column-major Mm x Md per frame
        if jacobian:
            return Vm, J.transpose(1, 2)
        return Vm

    def solve_complex(self, materialDistribution, options: SolveOptions | None = None, jacobian: bool = False,
                      raise_on_noconv: bool = True):
        """Forward solve for complex material values (complex64 CUDA tensor,
        frames x elements); returns complex64 voltages (frames x Mm x Md) and,
        if asked, the complex Jacobian (frames x rowsJ x E),
        mpf_eit_forward_complex."""
        import torch
        g = materialDistribution
        if not (isinstance(g, torch.Tensor) and g.is_cuda and g.dtype == torch.complex64):
            raise TypeError("materialDistribution must be a complex64 CUDA tensor")
        g = g.reshape(-1, self.mesh.elements.shape[0]).contiguous()
        F = g.shape[0]
        Mm, Md = self.info["meas_count"], self.info["drive_count"]
        V = torch.empty((F, Md, Mm), dtype=torch.complex64, device=g.device)
        J = None
        if jacobian:
            J = torch.empty((F, self.mesh.elements.shape[0], self.jacobian_rows), dtype=torch.complex64,
                            device=g.device)
        st = _ffi.SolveStats()
        o = (options or SolveOptions(solver="bicgstab")).c()
        status = lib().mpf_eit_forward_complex(self._h, F, ctypes.c_void_p(g.data_ptr()),
                                               ctypes.c_void_p(V.data_ptr()),
                                               ctypes.c_void_p(J.data_ptr() if J is not None else 0),
                                               ctypes.byref(o), ctypes.byref(st), _stream())
        self.last_stats = st
        if status != _ffi.MPF_OK and (raise_on_noconv or status != 4):
            check(status)
        if jacobian:
            return V.transpose(1, 2), J.transpose(1, 2)
        return V.transpose(1, 2)

    def fields(self, frames: int):
        """Potentials of the last solve: (frames, components, Md+Mm, data_rows)."""
        import torch
        dr = self.info["data_rows"]
        cols = self.info["drive_count"] + self.info["meas_count"]
        out = torch.empty((frames, self.components, cols, dr), dtype=torch.float32, device="cuda")
        check(lib().mpf_eit_fields(self._h, frames, ptr(out), _stream()))
        return out

    def fields_complex(self, frames: int):
        """Complex potentials of the last solve_complex: (frames, components,
        Md+Mm, data_rows) complex64 (mpf_eit_fields_complex)."""
        import torch
        dr = self.info["data_rows"]
        cols = self.info["drive_count"] + self.info["meas_count"]
        out = torch.empty((frames, self.components, cols, dr), dtype=torch.complex64, device="cuda")
        check(lib().mpf_eit_fields_complex(self._h, frames, ptr(out), _stream()))
        return out

    def gn_step(self, gamma, v_meas, lam: float, options: SolveOptions | None = None):
        """One regularised Gauss-Newton step in place on gamma; returns the
        relative data residual of each frame before the step."""
        import torch
        g, F = self._frames(gamma)
        if g.data_ptr() != gamma.data_ptr():
            raise ValueError("gamma must be contiguous")
        vm = self._vmeas(v_meas, F)
        res = np.zeros(F)
        st = _ffi.SolveStats()
        o = (options or SolveOptions()).c()
        check(lib().mpf_gn_step(self._h, F, ptr(g), ptr(vm), float(lam), ctypes.byref(o), ptr(res),
                                ctypes.byref(st), _stream()))
        self.last_stats = st
        return res

    def gn_solve(self, gamma, v_meas, lam: float, target: float = 1e-3, max_iters: int = 10,
                 options: SolveOptions | None = None):
        """Gauss-Newton until every frame's relative data residual <= target
        (mpf_gn_solve); gamma is updated in place.  Returns (updates per
        frame, final residual per frame, GnStats)."""
        g, F = self._frames(gamma)
        if g.data_ptr() != gamma.data_ptr():
            raise ValueError("gamma must be contiguous")
        vm = self._vmeas(v_meas, F)
        iters = np.zeros(F, np.int32)
        res = np.zeros(F)
        st = _ffi.GnStats()
        o = (options or SolveOptions()).c()
        check(lib().mpf_gn_solve(self._h, F, ptr(g), ptr(vm), float(lam), float(target), int(max_iters),
                                 ctypes.byref(o), ptr(iters), ptr(res), ctypes.byref(st), _stream()))
        return iters, res, st

    def learned_input(self, v_meas):
        """Network input of the learned warm start for (frames, Mm, Md)
        voltages: (V - V0) / rms(V0) per frame (mpf_eit_learned_input)."""
        import torch
        F = v_meas.shape[0]
        vm = self._vmeas(v_meas, F)
        x = torch.empty((F, vm.shape[1] * vm.shape[2]), dtype=torch.float32, device=vm.device)
        check(lib().mpf_eit_learned_input(self._h, F, ptr(vm), ptr(x), _stream()))
        return x

    def learned_prior(self, lam: float):
        """Sets the linear prior of the learned start (mpf_eit_learned_prior):
        the first Gauss-Newton update from the homogeneous distribution with
        regularisation lam, as a fixed linear map of the network input.
        lam = 0 removes it."""
        check(lib().mpf_eit_learned_prior(self._h, float(lam), _stream()))
        self.prior_lambda = float(lam) if lam else None

    def learned_prior_apply(self, x, out=None, mode: int = 0):
        """prior(x) for network inputs x (frames x L): into a new
        (frames x n_elements) tensor, or into `out` (mode 0 =, 1 +=, -1 -=)."""
        import torch
        if not (isinstance(x, torch.Tensor) and x.is_cuda and x.dtype == torch.float32 and x.dim() == 2):
            raise TypeError("x must be a (frames x inputs) float32 CUDA tensor")
        x = x.contiguous()
        E = self.mesh.elements.shape[0]
        if out is None:
            out = torch.empty((x.shape[0], E), dtype=torch.float32, device=x.device)
            mode = 0
        if out.dtype != torch.float32 or not out.is_contiguous() or out.shape[0] != x.shape[0] or out.shape[1] < E:
            raise ValueError("out must be a contiguous float32 (frames x >= n_elements) tensor")
        check(lib().mpf_eit_learned_prior_apply(self._h, x.shape[0], ptr(x), ptr(out), out.shape[1], int(mode),
                                                _stream()))
        return out

    def gn_solve_learned(self, net, v_meas, lam: float, target: float = 1e-3, max_iters: int = 10,
                         options: SolveOptions | None = None):
        """Gauss-Newton from the network's prediction (mpf_gn_solve_learned).
        Returns (gamma, updates per frame, final residual per frame, accepted
        per frame, GnStats)."""
        import torch
        F = v_meas.shape[0]
        vm = self._vmeas(v_meas, F)
        g = torch.empty((F, self.mesh.elements.shape[0]), dtype=torch.float32, device=vm.device)
        iters = np.zeros(F, np.int32)
        res = np.zeros(F)
        acc = np.zeros(F, np.int32)
        st = _ffi.GnStats()
        o = (options or SolveOptions()).c()
        check(lib().mpf_gn_solve_learned(self._h, net._h, F, ptr(g), ptr(vm), float(lam), float(target),
                                         int(max_iters), ctypes.byref(o), ptr(iters), ptr(res), ptr(acc),
                                         ctypes.byref(st), _stream()))
        return g, iters, res, acc, st

    REGULARIZATIONS = {"identity": 0, "noser": 1, "laplacian": 2}

    def inverse(self, jacobian, calculation, measurement, factor: float, regularization: str = "identity"):
        """One regularised inverse step (solver::Inverse, mpf_inverse_solve):
        (J^T J + (ref factor)^2 R) dsigma = J^T (measurement - calculation) for
        every image.  jacobian: (rowsJ, E) as returned by solve(jacobian=True)
        for one frame; calculation, measurement: (images, Mm, Md).  Returns
        dsigma (images, E)."""
        import torch
        if regularization not in self.REGULARIZATIONS:
            raise ValueError(f"regularization must be one of {sorted(self.REGULARIZATIONS)}")
        J = jacobian.reshape(self.jacobian_rows, -1).t().contiguous()  # reference layout storage (E, rowsJ)
        images = calculation.shape[0]
        calc = self._vmeas(calculation, images)
        meas = self._vmeas(measurement, images)
        out = torch.empty((images, self.mesh.elements.shape[0]), dtype=torch.float32, device=calc.device)
        check(lib().mpf_inverse_solve(self._h, self.REGULARIZATIONS[regularization], float(factor), images, ptr(J),
                                      ptr(calc), ptr(meas), ptr(out), _stream()))
        return out

    def inverse_complex(self, jacobian, calculation, measurement, factor: float, regularization: str = "identity"):
        """Complex regularised inverse step (solver::Inverse on
        thrust::complex<float>, mpf_inverse_solve_complex):
        (J^T J + (ref factor)^2 R) dsigma = J^T (measurement - calculation)
        with the plain transpose.  jacobian: complex64 (rowsJ, E) as returned
        by solve_complex(jacobian=True) for one frame; calculation,
        measurement: complex64 (images, Mm, Md).  Returns complex64 dsigma
        (images, E)."""
        import torch
        if regularization not in self.REGULARIZATIONS:
            raise ValueError(f"regularization must be one of {sorted(self.REGULARIZATIONS)}")
        for name, t in (("jacobian", jacobian), ("calculation", calculation), ("measurement", measurement)):
            if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.complex64):
                raise TypeError(f"{name} must be a complex64 CUDA tensor")
        J = jacobian.reshape(self.jacobian_rows, -1).t().contiguous()  # reference layout storage (E, rowsJ)
        images = calculation.shape[0]
        calc = self._vmeas(calculation, images)
        meas = self._vmeas(measurement, images)
        out = torch.empty((images, self.mesh.elements.shape[0]), dtype=torch.complex64, device=calc.device)
        vp = lambda t: ctypes.c_void_p(t.data_ptr())
        check(lib().mpf_inverse_solve_complex(self._h, self.REGULARIZATIONS[regularization], float(factor), images,
                                              vp(J), vp(calc), vp(meas), vp(out), _stream()))
        return out

    def group_iterations(self) -> np.ndarray:
        """CG iterations per (frame, active harmonic) group of the last inner solve."""
        out = np.zeros(65536, np.int32)
        cnt = ctypes.c_int32(0)
        check(lib().mpf_eit_group_iterations(self._h, ptr(out), out.size, ctypes.byref(cnt)))
        return out[:cnt.value].copy()

    def cg_variants(self, frames: int = 1, set=None) -> np.ndarray:
        """CG kernel variants {spmm, update, direction} a solve with `frames`
        frames uses; `set` fixes them (-1 = autotune), see mpf_eit_cg_variants."""
        get = np.zeros(3, np.int32)
        sv = None if set is None else np.ascontiguousarray(set, np.int32)
        check(lib().mpf_eit_cg_variants(self._h, None if sv is None else ptr(sv), int(frames), ptr(get)))
        return get

    def profile_fem(self, gamma, reps: int = 10):
        """Mean CUDA-event time (ms) and algorithmic bytes of one launch of
        the assembly and the Jacobian kernels (mpf_eit_profile_fem)."""
        g, F = self._frames(gamma)
        ms = np.zeros(2)
        by = np.zeros(2)
        check(lib().mpf_eit_profile_fem(self._h, F, ptr(g), int(reps), ptr(ms), ptr(by), _stream()))
        return ms, by

    PHASES = ("assembly", "cg_setup", "cg", "voltages", "jacobian", "gram", "cholesky", "update", "network",
              "prior", "host")

    def phase_times(self, enable=None):
        """Device milliseconds accumulated per phase of the forward and
        Gauss-Newton calls since the timer was last (re)started, and the
        number of top-level calls timed (mpf_eit_phase_times).  enable=True
        restarts the accumulation, False stops it, None leaves it running."""
        ms = np.zeros(len(self.PHASES))
        calls = ctypes.c_int64(0)
        flag = -1 if enable is None else int(bool(enable))
        check(lib().mpf_eit_phase_times(self._h, flag, ptr(ms), len(self.PHASES), ctypes.byref(calls)))
        return dict(zip(self.PHASES, ms.tolist())), int(calls.value)

    def profile_cg(self, gamma, reps: int = 20):
        """Mean CUDA-event time (ms) and algorithmic bytes of one launch of the
        SpMM, update and direction kernels (mpf_eit_profile_cg)."""
        g, F = self._frames(gamma)
        ms = np.zeros(3)
        by = np.zeros(3)
        check(lib().mpf_eit_profile_cg(self._h, F, ptr(g), int(reps), ptr(ms), ptr(by), _stream()))
        return ms, by

    def profile_cg_loop(self, gamma, graphs: int = 8):
        """Per-iteration ms of the CG loop as a solve runs it (graphs of 16
        iterations, host check between graphs), of its kernels launched one
        at a time, and host wall per iteration (mpf_eit_profile_cg_loop)."""
        g, F = self._frames(gamma)
        ms = np.zeros(3)
        check(lib().mpf_eit_profile_cg_loop(self._h, F, ptr(g), int(graphs), ptr(ms), _stream()))
        return {"loop_ms": float(ms[0]), "kernels_ms": float(ms[1]), "wall_ms": float(ms[2]),
                "outside_kernels_frac": float(1.0 - ms[1] / ms[0]) if ms[0] > 0 else None}


class SparseMatrix:
    """numeric::SparseMatrix on the GPU (mpf_sparse_*): built from the
    reference ELL layout (data_rows x 32 values and uint32 column ids,
    0xFFFFFFFF padding) or from a dense matrix; multiply() and solve() with
    CG or BiCGSTAB on column-major right-hand sides."""

    INVALID = 0xFFFFFFFF

    def __init__(self, values, column_ids, rows: int, density: int):
        import torch
        dr = data_rows(rows)
        v = torch.as_tensor(np.ascontiguousarray(values, np.float32).reshape(dr, 32)).cuda()
        c = torch.as_tensor(np.ascontiguousarray(column_ids, np.uint32).view(np.int32).reshape(dr, 32)).cuda()
        self.rows, self.density = int(rows), int(density)
        h = ctypes.c_void_p()
        check(lib().mpf_sparse_create(self.rows, ctypes.c_void_p(v.data_ptr()), ctypes.c_void_p(c.data_ptr()),
                                      self.density, ctypes.byref(h)))
        self._h = h

    @staticmethod
    def from_dense(A: np.ndarray) -> "SparseMatrix":
        """SparseMatrix(Matrix) of the reference: the nonzeros of each row in
        column order (src/numeric/sparse_matrix.cpp:137-160 via setValue)."""
        A = np.asarray(A, np.float64)
        n = A.shape[0]
        dr = data_rows(n)
        vals = np.zeros((dr, 32), np.float32)
        ids = np.full((dr, 32), SparseMatrix.INVALID, np.uint32)
        density = 0
        for i in range(n):
            nz = np.nonzero(A[i])[0]
            if len(nz) > 32:
                raise ValueError("mpFlow::numeric::SparseMatrix::setValue: sparse format full")
            vals[i, :len(nz)] = A[i, nz]
            ids[i, :len(nz)] = nz
            density = max(density, len(nz))
        return SparseMatrix(vals, ids, n, density)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            lib().mpf_sparse_destroy(h)
            self._h = None

    def multiply(self, x):
        """y = A x for a (rows x cols) float32 CUDA tensor."""
        import torch
        xc = x.reshape(self.rows, -1).t().contiguous()  # column-major storage
        y = torch.empty_like(xc)
        check(lib().mpf_sparse_multiply(self._h, ctypes.c_void_p(xc.data_ptr()), self.rows, xc.shape[0],
                                        ctypes.c_void_p(y.data_ptr()), self.rows, _stream()))
        return y.t()

    def solve(self, b, x0=None, solver: str = "cg", dc_free: bool = False, max_iter: int = 0, tol: float = 0.0):
        """x with A x = b for every column of a (rows x cols) float32 CUDA
        tensor; returns (x, iterations of the slowest column)."""
        import torch
        bc = b.reshape(self.rows, -1).t().contiguous()
        xc = torch.zeros_like(bc) if x0 is None else x0.reshape(self.rows, -1).t().contiguous().clone()
        it = ctypes.c_int32(0)
        check(lib().mpf_sparse_solve(self._h, SolveOptions.SOLVERS[solver], ctypes.c_void_p(bc.data_ptr()), self.rows,
                                     ctypes.c_void_p(xc.data_ptr()), self.rows, bc.shape[0], int(max_iter), float(tol),
                                     int(bool(dc_free)), ctypes.byref(it), _stream()))
        return xc.t(), it.value


class EITBatch:
    """Forward solves of several EIT models (meshes of uneven size, 16 or 32
    electrodes, one harmonic set) in the same CG launches (mpf_batch_*).

    ``solve`` takes one (frames x elements_i) float32 CUDA tensor per model
    and returns one (frames x Mm_i x Md_i) voltage tensor per model, equal to
    ``models[i].solve`` (cold start, Jacobi preconditioner)."""

    def __init__(self, models):
        self.models = list(models)
        handles = (ctypes.c_void_p * len(self.models))(*[m._h.value for m in self.models])
        h = ctypes.c_void_p()
        check(lib().mpf_batch_create(handles, len(self.models), ctypes.byref(h)))
        self._h = h
        self.last_stats = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            lib().mpf_batch_destroy(h)
            self._h = None

    def solve(self, gammas, options: SolveOptions | None = None, raise_on_noconv: bool = True):
        """Forward solves of every model's frames in the same launches
        (mpf_batch_forward): gammas is one (frames x elements) float32 CUDA
        tensor per model, all with the same frame count.  Returns each
        model's voltages (frames x Mm x Md)."""
        import torch
        if len(gammas) != len(self.models):
            raise ValueError(f"expected {len(self.models)} material tensors, got {len(gammas)}")
        gs, Vs = [], []
        F = None
        for m, g in zip(self.models, gammas):
            gg, Fi = m._frames(g)
            if F is not None and Fi != F:
                raise ValueError("every model needs the same number of frames")
            F = Fi
            gs.append(gg)
            Vs.append(torch.empty((F, m.info["drive_count"], m.info["meas_count"]), dtype=torch.float32,
                                  device=gg.device))
        gp = (ctypes.c_void_p * len(gs))(*[g.data_ptr() for g in gs])
        vp = (ctypes.c_void_p * len(Vs))(*[v.data_ptr() for v in Vs])
        st = _ffi.SolveStats()
        o = (options or SolveOptions()).c()
        status = lib().mpf_batch_forward(self._h, F, gp, vp, ctypes.byref(o), ctypes.byref(st), _stream())
        self.last_stats = st
        if status != _ffi.MPF_OK and (raise_on_noconv or status != 4):
            check(status)
        return [v.transpose(1, 2) for v in Vs]

    def iterations(self, frames: int) -> np.ndarray:
        """CG iterations of the last solve, shape (models, frames, active harmonics)."""
        out = np.zeros(len(self.models) * frames * 128, np.int32)
        cnt = ctypes.c_int32(0)
        check(lib().mpf_batch_iterations(self._h, ptr(out), out.size, ctypes.byref(cnt)))
        return out[:cnt.value].reshape(len(self.models), frames, -1).copy()

    def cg_stats(self):
        """(device ms, algorithmic bytes) of the last solve's CG."""
        ms, by = ctypes.c_double(0), ctypes.c_double(0)
        check(lib().mpf_batch_cg_stats(self._h, ctypes.byref(ms), ctypes.byref(by)))
        return ms.value, by.value

    def cg_variants(self, frames: int = 1, set=None) -> np.ndarray:
        """Launch-shape codes per width class (rows) and kernel (columns)."""
        get = np.zeros(12, np.int32)
        ncl = ctypes.c_int32(0)
        sv = None if set is None else np.ascontiguousarray(set, np.int32)
        check(lib().mpf_batch_cg_variants(self._h, None if sv is None else ptr(sv), int(frames), ptr(get), get.size,
                                          ctypes.byref(ncl)))
        return get[:3 * ncl.value].reshape(-1, 3).copy()


def gram_split_bf16(A):
    """C = A A^T (rows x rows) for a batch of row-major float32 CUDA matrices."""
    import torch
    if A.dim() == 2:
        A = A[None]
    B, rows, cols = A.shape
    A = A.contiguous()
    C = torch.empty((B, rows, rows), dtype=torch.float32, device=A.device)
    check(lib().mpf_gram_split_bf16(B, rows, cols, ptr(A), cols, ptr(C), _stream()))
    return C


def profile_gram(batch: int, rows: int, cols: int, reps: int = 5) -> float:
    """Device milliseconds of one J J^T of the GN step (mpf_profile_gram)
    for batch x (rows x cols) operands."""
    ms = ctypes.c_double(0.0)
    check(lib().mpf_profile_gram(int(batch), int(rows), int(cols), int(reps), ctypes.byref(ms), _stream()))
    return ms.value


def cholesky_solve_f64(A, Bm, shift: float = 0.0):
    """Solve (A + shift I) X = B for batches of float64 CUDA matrices (A overwritten)."""
    import torch
    if A.dim() == 2:
        A, Bm = A[None], Bm[None]
    batch, n, _ = A.shape
    nrhs = Bm.shape[1] if Bm.dim() == 3 else 1
    info = torch.zeros(batch, dtype=torch.int32, device=A.device)
    check(lib().mpf_cholesky_solve_f64(batch, n, ptr(A), float(shift), ptr(Bm), nrhs, ptr(info), _stream()))
    return info
