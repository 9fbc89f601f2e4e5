"""Step graphs and concurrent group streams change launch mechanics only.

Steady-state steps are replayed from CUDA graphs (one per ring-buffer
phase) and batches with several operator keys step their groups on
separate streams.  Both must give bit-identical results to direct launches
on one stream, and the launch counter must count the replayed kernels.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ("T", "omg", "up", "ur", "psi")

CASES = [("CNAB2", 17, 8, 1e4, 1e-4, 11), ("SBDF3", 33, 20, 1e5, 1e-5, 12),
         ("SBDF4", 17, 10, 1e4, 1e-5, 13), ("ARS443", 17, 10, 1e4, 1e-5, 14),
         ("ARS343", 17, 10, 1e4, 1e-5, 15), ("SBDF3", 33, 20, 3e5, 1e-5, 16),
         ("CB4", 17, 10, 1e4, 1e-5, 17), ("KC885", 17, 8, 1e4, 1e-5, 18)]


def run(fg, graphs, nsteps):
    prev = fg.set_step_graphs(graphs)
    try:
        b = fg.Batch([fg.make_params(R, Nm, s, ra=ra, dt=dt) for s, R, Nm, ra, dt, _ in CASES])
        b.init_noise([c[-1] for c in CASES])
        n0 = fg.launch_count()
        b.step(nsteps)
        launches = fg.launch_count() - n0
        states = [b.get_state(i) for i in range(len(CASES))]
        diags = b.diagnostics()
        b.close()
    finally:
        fg.set_step_graphs(prev)
    return states, diags, launches


def test_graph_replay_is_bit_identical_to_direct_launches(fg):
    nsteps = 13  # several passes over every ring phase (period <= 4)
    # a first run lets the contraction autotuner measure every shape, so
    # that both runs below take the same paths and launch the same kernels
    run(fg, False, 2)
    direct, d_diag, n_direct = run(fg, False, nsteps)
    graph, g_diag, n_graph = run(fg, True, nsteps)
    for i, (a, b) in enumerate(zip(direct, graph)):
        for f in FIELDS:
            assert np.array_equal(a[f], b[f]), (CASES[i][0], f)
    for a, b in zip(d_diag, g_diag):
        assert a == b
    # every kernel of a replayed step is still counted
    assert n_graph == n_direct


def test_graph_replay_after_reset_and_new_state(fg):
    p = fg.make_params(17, 8, "SBDF3", ra=1e4, dt=1e-4)
    g = fg.Instance(p)
    g.init_noise(3)
    g.step(7)
    g.init_noise(4)  # histories restart: the first step runs directly again
    g.step(9)
    s1 = g.get_state()
    prev = fg.set_step_graphs(False)
    try:
        h = fg.Instance(p)
        h.init_noise(4)
        h.step(9)
        s2 = h.get_state()
    finally:
        fg.set_step_graphs(prev)
    for f in FIELDS:
        assert np.array_equal(s1[f], s2[f]), f


@pytest.mark.parametrize("R,Nm,scheme,dt,nb", [
    # Np = 510 (radix 2, 3, 5, 17): one instance (65 lines) runs the
    # block-per-line pass, five (325 lines) the warp-per-line one
    (65, 170, "SBDF3", 1e-6, 5),
    # Np = 1023 (radix 3, 11, 31): one instance with 8 warps per line, three
    # (291 lines) with 4; longer batches keep the block-per-line form here
    # (it holds 16 warps per SM against 4)
    (97, 341, "ARS443", 1e-7, 3),
])
def test_block_per_line_and_warp_per_line_transforms_agree_bitwise(fg, fixed_paths, R, Nm, scheme, dt, nb):
    p = fg.make_params(R, Nm, scheme, ra=1e6, dt=dt)
    alone = fg.Instance(p)
    alone.init_noise(9)
    alone.step(3)
    b = fg.Batch([p] * nb)
    b.init_noise(list(range(9, 9 + nb)))
    b.step(3)
    sa, sb = alone.get_state(), b.get_state(0)
    for f in FIELDS:
        assert np.array_equal(sa[f], sb[f]), f
