"""Splitting independent cases over ranks (the batch study on several GPUs):
every case on exactly one rank, loads balanced by the greedy rule, and ranks
that mesh only their share get the same cases as a single process."""
import numpy as np

from fvdbm_jax_gb300 import cases as CS


def test_partition_covers_every_case_once_and_balances():
    rng = np.random.default_rng(0)
    costs = rng.uniform(2e3, 1.2e5, 256)
    for n in (1, 2, 3, 8):
        parts = CS.partition_cases(costs, n)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(costs.size))
        loads = [costs[p].sum() for p in parts]
        # greedy LPT: no rank exceeds the mean by more than the largest case
        assert max(loads) <= costs.sum() / n + costs.max()


def test_rank_subsets_match_the_full_suite():
    full, dfull = CS.batch_suite(seed=3, n_cavity=3, n_porous=3, cavity_cells=(2000, 4000),
                                 porous_cells=(3000, 5000), obstacles=(5, 10))
    key = lambda d: (d["kind"], round(d["re"], 9), d["cells"])
    seen = []
    for r in range(2):
        sub, dsub = CS.batch_suite(seed=3, n_cavity=3, n_porous=3, cavity_cells=(2000, 4000),
                                   porous_cells=(3000, 5000), obstacles=(5, 10), rank=r, n_ranks=2)
        seen += [key(d) for d in dsub]
    assert sorted(seen) == sorted(key(d) for d in dfull)


def test_lattice_unit_scales_give_unit_spacing():
    """Cases meshed in lattice units have a mesh spacing of about 1, and
    their tau follows the notebooks' rule with L the side in cells."""
    from fvdbm_jax_gb300 import cases as CS
    import numpy as np
    sc = CS.cavity_lattice_scale(21)
    dyn, c, f, n, m = CS.lid_cavity(21, 0.6, scale=sc, mesher=True)
    L = np.asarray(m.face_lengths)
    assert sc == 20.0 and 0.8 < np.median(L) < 1.2
    assert abs(float(dyn.delta_t) - 0.5 * L.min()) < 1e-6
    sp = CS.porous_lattice_scale(6000, 0.8)
    dyn, c, f, n, m = CS.porous_square(20, 6000, 0.6, porosity=0.8, scale=sp, mesher=True, seed=3)
    L = np.asarray(m.face_lengths)
    assert 0.7 < np.median(L) < 1.3, np.median(L)
    suite, desc = CS.batch_suite(seed=1, n_cavity=2, n_porous=1, cavity_cells=(2000, 3000),
                                 porous_cells=(6000, 7000), obstacles=(20, 30), units="lattice")
    for d in desc:
        assert d["scale"] > 10
        assert abs(d["tau"] - (3 * CS.LID_U * d["scale"] / d["re"] + 0.5)) < 1e-12
