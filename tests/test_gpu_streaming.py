"""Streaming Tet4 assembly on the GPU (``-m gpu``): the scenarios of the reference's
``tests/test_reference_streaming.py`` restated on this library.

A pool of three copies of five original nodes holds up to six tets.  After
``prepare_tetrahedral_updates`` each edit goes through ``refresh_topology`` on fixed
device storage.  The assembled matrix, the preconditioner, the operator and the
elastic predictor must equal those of a solver built fresh on the edited model
(rtol 3e-5, atol 3e-6, the reference's bar).  The lineage counters follow
streaming.py:20-129.  Rejected edits leave the assembly untouched, and a graph
captured before the edits replays after them.
"""

import numpy as np
import pytest
import torch
from gpu_helpers import DEVICE, tensor, to_np

from newton_solver_fem_gb300 import SolverFEM, _lib, model_from_arrays

pytestmark = pytest.mark.gpu

ORIGINAL = 5
CAPACITY = 6
CORNERS = np.asarray(((0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1), (0.2, 0.3, -1)), dtype=np.float32)
INITIAL = ((0, (0, 1, 2, 3), 1.0), (1, (0, 2, 1, 4), 1.0))
SPLIT = ((1, (0, 2, 1, 4), 1.0), (0, (5, 6, 7, 8), 0.6), (0, (0, 1, 2, 3), 0.4))


@pytest.fixture(autouse=True)
def _cuda(cuda_device):
    yield


def edit(model, weights, records):
    """Write the records into the model's arrays in place (slot, family, connectivity, material fraction)."""
    indices = np.zeros((CAPACITY, 4), np.int32)
    poses = np.tile(np.eye(3), (CAPACITY, 1, 1))
    materials = np.zeros((CAPACITY, 3))
    fractions = np.zeros(CAPACITY)
    masses = np.zeros(model.particle_count)
    rest = np.tile(CORNERS, (3, 1)).astype(np.float64)
    for slot, (family, connectivity, fraction) in enumerate(records):
        nodes = list(connectivity)
        edges = (rest[nodes[1:]] - rest[nodes[0]]).T
        if np.linalg.det(edges) < 0:
            nodes[1], nodes[2] = nodes[2], nodes[1]
            edges = (rest[nodes[1:]] - rest[nodes[0]]).T
        indices[slot] = nodes
        poses[slot] = np.linalg.inv(edges)
        materials[slot] = fraction * np.asarray((1000.0 + 300.0 * family, 1500.0 + 200.0 * family, 0.0))
        fractions[slot] = fraction
        masses[nodes] += fraction * 200.0 * np.linalg.det(edges) / 24.0
    model.tet_indices.copy_(torch.tensor(indices, device=DEVICE))
    model.tet_poses.copy_(tensor(poses))
    model.tet_materials.copy_(tensor(materials))
    weights.copy_(tensor(fractions))
    model.particle_mass.copy_(tensor(np.where(masses > 0, masses, 1.0)))
    model.particle_inv_mass.copy_(tensor(np.divide(1.0, masses, out=np.zeros_like(masses), where=masses > 0)))
    model.particle_flags.copy_(torch.tensor((masses > 0).astype(np.int32), device=DEVICE))


def make_model(records=INITIAL):
    x = np.tile(CORNERS, (3, 1))
    model = model_from_arrays(x, np.ones(len(x)), gravity=(0.0, 0.0, -9.81), device=DEVICE)
    model.tet_indices = torch.zeros((CAPACITY, 4), dtype=torch.int32, device=DEVICE)
    model.tet_poses = tensor(np.tile(np.eye(3), (CAPACITY, 1, 1)))
    model.tet_materials = torch.zeros((CAPACITY, 3), dtype=torch.float32, device=DEVICE)
    model.tet_activations = torch.zeros(CAPACITY, dtype=torch.float32, device=DEVICE)
    weights = torch.zeros(CAPACITY, dtype=torch.float32, device=DEVICE)
    edit(model, weights, records)
    return model, weights


def make_solver(model, weights, streaming=False):
    solver = SolverFEM(model, tet_volume_weights=weights, dt=1.0 / 120, solver_type="cg",
                       preconditioner_type="block_diag", linear_solver_maxiter=30, self_contact_ke=0.0)
    if streaming:
        solver.prepare_tetrahedral_updates(ORIGINAL)
    return solver


def deformed(model):
    p = to_np(model.particle_q).copy()
    p[:, 0] += 0.17 * p[:, 2]
    p[:, 1] -= 0.08 * p[:, 0]
    p[:, 2] *= 0.91
    return tensor(p)


def sources(entries):
    values = np.full(CAPACITY, -1, np.int32)
    values[: len(entries)] = entries
    return torch.tensor(values, device=DEVICE)


def apply_operator(solver, x):
    y = torch.empty_like(x)
    _lib.check(_lib.load().fem_apply_operator(solver._handle, x.data_ptr(), y.data_ptr(),
                                              torch.cuda.current_stream().cuda_stream))
    return y


def check_matrix(solver, positions, records):
    model, weights = make_model(records)
    reference = make_solver(model, weights)
    reference.refresh_tangent(positions)
    expected = reference.A_bsr.dense()
    np.testing.assert_allclose(solver.A_bsr.dense(), expected, rtol=3e-5, atol=3e-6)
    np.testing.assert_allclose(to_np(solver._pc_inv_diag), to_np(reference._pc_inv_diag), rtol=3e-5, atol=3e-6)
    rng = np.random.default_rng(725)
    x = tensor(rng.normal(size=(model.particle_count, 3)))
    np.testing.assert_allclose(to_np(apply_operator(solver, x)), (expected @ to_np(x).ravel()).reshape(-1, 3),
                               rtol=3e-5, atol=4e-6)
    # the elastic predictor sum_j A_ij (v_j - v_i) of a prepared step, against the fresh solver's
    state = model.state()
    state.particle_q.copy_(positions)
    state.particle_qd.copy_(x)
    got = solver.prepare_step(state, None, None, solver.dt)._predictor.clone()
    want = reference.prepare_step(state, None, None, reference.dt)._predictor
    np.testing.assert_allclose(to_np(got), to_np(want), rtol=3e-5, atol=4e-6)


def test_split_shuffled_lineage_shared_edge_removal():
    model, weights = make_model()
    solver = make_solver(model, weights, streaming=True)
    nnzb = solver.matrix_info()["nnzb"]
    positions = deformed(model)
    solver.refresh_tangent(positions)
    check_matrix(solver, positions, INITIAL)

    edit(model, weights, SPLIT)
    solver.refresh_topology(positions, element_sources=sources((1, 0, 0)))
    check_matrix(solver, positions, SPLIT)
    u = solver._streaming.last_update
    assert (u["dirty_elements"], u["reused_elements"], u["active_elements"]) == (2, 1, 3)

    # the removed child shares three original nodes with the retained tet: its
    # contribution vanishes without erasing the retained stiffness
    retained = SPLIT[:2]
    edit(model, weights, retained)
    solver.refresh_topology(positions)
    check_matrix(solver, positions, retained)
    u = solver._streaming.last_update
    assert (u["dirty_elements"], u["removed_elements"]) == (0, 1)

    edit(model, weights, ())
    solver.refresh_topology(positions)
    check_matrix(solver, positions, ())
    assert solver._streaming.last_update["active_elements"] == 0
    assert solver.matrix_info()["nnzb"] == nnzb  # the reserved pattern never changes
    state, output = model.state(), model.state()
    solver.step(state, output, model.control(), None, solver.dt)
    np.testing.assert_array_equal(to_np(output.particle_q), to_np(state.particle_q))
    np.testing.assert_array_equal(to_np(output.particle_qd), 0.0)


def test_moved_unchanged_tet_refreshes_current_tangent():
    model, weights = make_model()
    solver = make_solver(model, weights, streaming=True)
    positions = deformed(model)
    solver.refresh_tangent(positions)
    moved = to_np(positions)
    moved[4] += (0.15, -0.05, 0.09)
    positions = tensor(moved)
    solver.refresh_topology(positions)
    check_matrix(solver, positions, INITIAL)
    u = solver._streaming.last_update
    assert (u["dirty_elements"], u["reused_elements"], u["touched_rows"]) == (1, 1, 0)
    assert (u["topology_inserted_elements"], u["topology_removed_elements"]) == (0, 0)


def test_element_rebuild_keeps_the_reserved_pattern():
    model, weights = make_model()
    solver = make_solver(model, weights, streaming=True)
    info = solver.matrix_info()
    columns = solver.A_bsr.columns.clone()
    positions = deformed(model)
    solver.rebuild_element_blocks(positions, solver.dt)
    assert solver.matrix_info() == info
    assert torch.equal(solver.A_bsr.columns, columns)
    check_matrix(solver, positions, INITIAL)


def test_reject_unreserved_edge_without_mutating_assembly():
    model, weights = make_model()
    solver = make_solver(model, weights, streaming=True)
    positions = deformed(model)
    solver.refresh_tangent(positions)
    saved = (solver.A_bsr.dense(), to_np(solver._pc_inv_diag), solver.bsr_values.clone())
    edit(model, weights, ((0, (0, 1, 3, 4), 1.0),))  # original nodes 3 and 4 never shared a tet
    with pytest.raises(ValueError, match="outside the reserved"):
        solver.refresh_topology(positions)
    np.testing.assert_array_equal(solver.A_bsr.dense(), saved[0])
    np.testing.assert_array_equal(to_np(solver._pc_inv_diag), saved[1])
    assert torch.equal(solver.bsr_values, saved[2])
    edit(model, weights, INITIAL)
    solver.refresh_topology(positions)
    check_matrix(solver, positions, INITIAL)
    assert solver._streaming.last_update["dirty_elements"] == 0


def test_invalid_source_rejected_before_assembly_changes():
    model, weights = make_model()
    solver = make_solver(model, weights, streaming=True)
    positions = deformed(model)
    solver.refresh_tangent(positions)
    expected = solver.A_bsr.dense()
    with pytest.raises(ValueError, match="source"):
        solver.refresh_topology(positions, element_sources=sources((CAPACITY, 1)))
    np.testing.assert_array_equal(solver.A_bsr.dense(), expected)
    with pytest.raises(ValueError):
        solver.refresh_topology(positions, element_sources=torch.zeros(2, dtype=torch.int32, device=DEVICE))


def test_preparation_rules():
    model, weights = make_model()
    solver = make_solver(model, weights, streaming=True)
    with pytest.raises(RuntimeError, match="already prepared"):
        solver.prepare_tetrahedral_updates(ORIGINAL)
    with pytest.raises(ValueError, match="construction timestep"):
        solver.refresh_tangent(model.particle_q, solver.dt / 2)
    other = make_solver(*make_model())
    with pytest.raises(ValueError, match="whole copies"):
        other.prepare_tetrahedral_updates(4)
    stepped = make_solver(*make_model())
    s0, s1 = model.state(), model.state()
    stepped.step(s0, s1, None, None, stepped.dt)
    with pytest.raises(RuntimeError, match="before capturing or stepping"):
        stepped.prepare_tetrahedral_updates(ORIGINAL)


def test_original_capture_replays_after_multiple_edits():
    model, weights = make_model()
    solver = make_solver(model, weights, streaming=True)
    state, output = model.state(), model.state()
    state.particle_q.copy_(deformed(model))
    state.particle_qd.copy_(state.particle_q * tensor([0.1, -0.05, 0.02]))
    solver.refresh_tangent(state.particle_q)
    solver.step(state, output, None, None, solver.dt)
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    stream = torch.cuda.Stream()
    stream.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(stream):
        with torch.cuda.graph(graph, stream=stream):
            solver.refresh_tangent(state.particle_q)
            solver.step(state, output, None, None, solver.dt)
    torch.cuda.current_stream().wait_stream(stream)
    for records, srcs in ((SPLIT, (1, 0, 0)), (SPLIT[:2], (0, 1))):
        edit(model, weights, records)
        solver.refresh_topology(state.particle_q, element_sources=sources(srcs))
        graph.replay()
        torch.cuda.synchronize()
        ref_model, ref_weights = make_model(records)
        reference = make_solver(ref_model, ref_weights)
        expected = ref_model.state()
        reference.refresh_tangent(state.particle_q)
        reference.step(state, expected, None, None, reference.dt)
        np.testing.assert_allclose(to_np(output.particle_q), to_np(expected.particle_q), rtol=2e-5, atol=2e-6)
        np.testing.assert_allclose(to_np(output.particle_qd), to_np(expected.particle_qd), rtol=1e-4, atol=2e-5)
