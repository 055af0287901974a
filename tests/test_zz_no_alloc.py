"""The allocation-free PCG entry point agrees with the handle path (``-m gpu``).

``fem_pcg_solve_noalloc`` serves callers that cannot call cudaMalloc while they
run (a host application that owns all device memory, or a loop that cannot take
an allocation's implicit synchronisation): it keeps its working vectors in a
static device array instead of allocating.  This test solves the same systems
the handle path (``fem_step``) solved on two substeps in a row -- the exported
matrix and the step's final right-hand side, from the same warm start -- and
compares the solutions at the parity bar used for solves (1e-4 relative L2).
This file is collected last so that a failure here comes after every other test.
"""

import ctypes

import numpy as np
import pytest
import torch

from newton_solver_fem_gb300 import SolverFEM, _lib, build, model_from_arrays, scenes

pytestmark = pytest.mark.gpu


def _solve_noalloc(lib, A, rhs, x, rows, tol, maxiter, info):
    code = lib.fem_pcg_solve_noalloc(A.offsets.data_ptr(), A.columns.data_ptr(), A.values.data_ptr(),
                                     rhs.data_ptr(), x.data_ptr(), rows, tol, maxiter, info.data_ptr(),
                                     torch.cuda.current_stream().cuda_stream)
    _lib.check(code, "fem_pcg_solve_noalloc")
    torch.cuda.synchronize()


def test_noalloc_solve_matches_handle_path_on_two_substeps(cuda_device):
    build.build()
    lib = _lib.load()
    sc = scenes.tet_jittered_48(n=6)  # 343 nodes, Tet4 + edge springs, no fixed nodes
    model = model_from_arrays(sc.x, sc.mass, tets=sc.tets, tet_materials=sc.tet_materials, springs=sc.springs,
                              spring_ke=sc.spring_ke, spring_kd=sc.spring_kd, gravity=sc.gravity, device=cuda_device)
    tol, maxiter = 1.0e-6, 400
    solver = SolverFEM(model, dt=sc.dt, solver_type="cg", preconditioner_type="block_diag", self_contact_ke=0.0,
                       linear_solver_tolerance=tol, linear_solver_maxiter=maxiter)
    A = solver.A_bsr
    rows = model.particle_count
    info = torch.zeros(2, dtype=torch.int32, device=cuda_device)
    s0, s1 = model.state(), model.state()
    s0.particle_qd.copy_(0.05 * torch.randn_like(s0.particle_qd))
    warm = torch.zeros((rows, 3), dtype=torch.float32, device=cuda_device)
    for _ in range(2):  # two calls in a row, the second from the first solution as warm start
        solver.step(s0, s1, None, None, sc.dt)
        torch.cuda.synchronize()
        expected = solver.velocity_increment.clone()
        x = warm.clone()
        _solve_noalloc(lib, A, s0.particle_f, x, rows, tol, maxiter, info)
        got = x.cpu().numpy().astype(np.float64)
        want = expected.cpu().numpy().astype(np.float64)
        assert int(info[1]) == 0
        assert int(info[0]) > 0
        assert np.isfinite(got).all()
        assert np.linalg.norm(got - want) / np.linalg.norm(want) < 1e-4
        warm = expected
        s0, s1 = s1, s0


def test_noalloc_rejects_sizes_beyond_its_static_capacity(cuda_device):
    lib = _lib.load()
    code = lib.fem_pcg_solve_noalloc(None, None, None, None, None, 65537, 1e-2, 10, None, None)
    assert code == _lib.FEM_ERR_BAD_ARG


def _chain_system(rows, device):
    """A block tridiagonal SPD system (4I on the diagonal, -I to each neighbour) in BSR form."""
    import numpy as np

    offsets, columns, values = [0], [], []
    for i in range(rows):
        for j in (i - 1, i, i + 1):
            if 0 <= j < rows:
                columns.append(j)
                values.append(4.0 * np.eye(3) if j == i else -np.eye(3))
        offsets.append(len(columns))

    class A:
        pass

    a = A()
    a.offsets = torch.tensor(offsets, dtype=torch.int32, device=device)
    a.columns = torch.tensor(columns, dtype=torch.int32, device=device)
    a.values = torch.tensor(np.asarray(values), dtype=torch.float32, device=device)
    return a


def test_noalloc_bounded_wait_reports_timeout_in_info_and_recovers(cuda_device, monkeypatch):
    """A grid-barrier wait that runs out (zero wait limit) still writes info: status bit 1 is set and the
    kernel returns.  With the default limit the next call on the same context solves the system."""
    lib = _lib.load()
    rows = 60_000  # hundreds of co-resident CTAs, so some CTA reaches the first barrier before the others
    A = _chain_system(rows, cuda_device)
    g = torch.Generator(device=cuda_device).manual_seed(7)
    rhs = torch.randn((rows, 3), device=cuda_device, generator=g)
    info = torch.full((2,), -1, dtype=torch.int32, device=cuda_device)
    x = torch.zeros((rows, 3), dtype=torch.float32, device=cuda_device)
    monkeypatch.setenv("FEM_NOALLOC_WAIT_LIMIT_NS", "0")
    _solve_noalloc(lib, A, rhs, x, rows, 1e-6, 100, info)
    assert int(info[1]) & 1
    monkeypatch.delenv("FEM_NOALLOC_WAIT_LIMIT_NS")
    for _ in range(2):  # the context stays usable: two solves in a row at the default limit
        x = torch.zeros((rows, 3), dtype=torch.float32, device=cuda_device)
        _solve_noalloc(lib, A, rhs, x, rows, 1e-6, 100, info)
        assert int(info[1]) == 0
        xs, bs = x.double().cpu(), rhs.double().cpu()
        ax = 4.0 * xs
        ax[1:] -= xs[:-1]
        ax[:-1] -= xs[1:]
        assert float((ax - bs).norm() / bs.norm()) < 1e-5
