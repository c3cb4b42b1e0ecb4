"""Synthetic workload generators: seeded and deterministic, and at the sizes
and porosity the throughput configurations state (porous square: 400
obstacles, porosity 0.70 +- 0.01; channel with cylinder: about 60k
triangles)."""
import numpy as np


def test_porous_square_is_seeded_and_hits_the_porosity():
    from fvdbm_jax_gb300 import Mesher, meshgen
    raw = meshgen.porous(n_obstacles=400, n_target=100_000, porosity=0.70, seed=0)
    again = meshgen.porous(n_obstacles=400, n_target=100_000, porosity=0.70, seed=0)
    assert np.array_equal(raw.points, again.points) and np.array_equal(raw.elements, again.elements)
    other = meshgen.porous(n_obstacles=400, n_target=100_000, porosity=0.70, seed=1)
    assert raw.points.shape != other.points.shape or not np.array_equal(raw.points, other.points)
    m = Mesher().import_meshpy(raw)
    m.calc_mesh_properties()
    assert 90_000 <= len(m.cells) <= 110_000
    assert abs(float(np.sum(m.cell_areas)) - 0.70) <= 0.01  # fluid area of the unit square


def test_channel_with_cylinder_size():
    from fvdbm_jax_gb300 import meshgen
    raw = meshgen.channel_cylinder(seed=0)
    assert 50_000 <= len(raw.elements) <= 70_000
