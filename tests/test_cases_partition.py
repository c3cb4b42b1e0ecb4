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
