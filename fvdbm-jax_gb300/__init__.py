"""fvdbm_jax_gb300: a GB300-native FVDBM time stepper that is a drop-in for
the ``Environment.init``/``Environment.step`` path of MADALERAU/FVDBM-JAX.

    from fvdbm_jax_gb300 import D2Q9, Mesher, Environment, meshgen

    mesher = Mesher().import_meshpy(meshgen.cavity())
    mesher.calc_mesh_properties()
    cells, faces, nodes = mesher.to_env(D2Q9(tau=0.6, delta_t=dt), "upwind")
    nodes = mesher.set_vel_node(nodes, 3, (0.1, 0.0))
    env = Environment(cells, faces, nodes); env.init()
    env = env.step()
"""
from .dynamics import D2Q9, D2Q13
from .containers import Cells, Faces, Nodes
from .mesher import Mesher
from .environment import Environment
from .batch import Batch
from . import meshgen

__all__ = ["D2Q9", "D2Q13", "Cells", "Faces", "Nodes", "Mesher", "Environment", "Batch", "meshgen"]
