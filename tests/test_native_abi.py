"""The C-ABI library builds for sm_103a, loads, exports every entry point
that include/*.h declares, and rejects invalid containers in host-side
validation (which runs before any CUDA call, so no GPU is needed)."""
import ctypes as C
import glob
import os
import re

import numpy as np
import pytest

from fvdbm_jax_gb300 import _native as nat

HEADERS = sorted(glob.glob(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                                        "*.h")))


def declared():
    src = "".join(open(h).read() for h in HEADERS)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\**\s*(fvdbm_\w+)\s*\(", src, re.M)))


def test_header_declares_the_boundary():
    names = declared()
    for n in ("fvdbm_create", "fvdbm_step", "fvdbm_set_state", "fvdbm_get_cells", "fvdbm_destroy",
              "fvdbm_batch_create", "fvdbm_residual", "fvdbm_mp_dense_fwd", "fvdbm_mp_adam"):
        assert n in names


def test_library_exports_every_declared_symbol():
    L = nat.lib()
    for n in declared():
        assert hasattr(L, n), n
    assert L.fvdbm_abi_version() == 4


def test_kernel_family_constants_match_the_header():
    src = open(os.path.join(os.path.dirname(HEADERS[0]), "fvdbm.h")).read()
    defs = {k: int(v) for k, v in re.findall(r"#define FVDBM_(KERNEL_\w+)\s+(\d+)", src)}
    assert defs["KERNEL_FAST"] == 9
    for k, v in defs.items():
        if hasattr(nat, k):
            assert getattr(nat, k) == v, k
    from fvdbm_jax_gb300.environment import _KERNEL
    assert _KERNEL["fast"] == defs["KERNEL_FAST"]
    assert _KERNEL["fused_nodes"] == defs["KERNEL_FUSED_NODES"]


def _tiny_mesh(**over):
    # two triangles sharing face 0; faces 1-4 are boundary faces
    a = dict(
        cfi=np.array([[0, 1, 2], [0, 3, 4]], np.int32), cfs=np.array([[1, 1, 1], [-1, 1, 1]], np.int32),
        fc=np.array([[0, 1], [0, -1], [0, -1], [1, -1], [1, -1]], np.int32),
        fd=np.full((5, 2), 0.1, np.float32), fnd=np.array([[0, 1], [1, 2], [2, 0], [1, 3], [3, 0]], np.int32),
        fn=np.tile(np.array([[1.0, 0.0]], np.float32), (5, 1)), fL=np.ones(5, np.float32),
        nt=np.array([1, 1, 1, 1], np.int32), nc=np.array([[0, 1], [0, 1], [0, -1], [1, -1]], np.int32),
        nd=np.array([[0.3, 0.3], [0.3, 0.3], [0.3, -1], [0.3, -1]], np.float32))
    a.update(over)
    return a


def _create(a, scheme=0, kernel=0):
    L = nat.lib()
    m = nat.Mesh(a["cfi"].shape[0], a["fc"].shape[0], a["nt"].shape[0], a["cfi"].shape[1], a["nc"].shape[1],
                 nat.iptr(a["cfi"]), nat.iptr(a["cfs"]), nat.iptr(a["fc"]), nat.fptr(a["fd"]), nat.iptr(a["fnd"]),
                 nat.fptr(a["fn"]), nat.fptr(a["fL"]), None, nat.iptr(a["nt"]), nat.iptr(a["nc"]),
                 nat.fptr(a["nd"]), None, None)
    p = nat.Params(scheme, 0, 1.0, 0.1, 1 / 3, 2 / 9, 2 / 3, 0, kernel, 0)
    h = C.c_void_p()
    rc = L.fvdbm_create(C.byref(m), C.byref(p), C.byref(h))
    if rc == 0:
        L.fvdbm_destroy(h)
    return rc, (L.fvdbm_last_error(None) or b"").decode()


@pytest.mark.parametrize("over,needle", [
    ({"cfi": np.array([[0, 1, 9], [0, 3, 4]], np.int32)}, "face_indices"),
    ({"cfs": np.array([[1, 2, 1], [-1, 1, 1]], np.int32)}, "face_normals"),
    ({"fc": np.array([[0, 7], [0, -1], [0, -1], [1, -1], [1, -1]], np.int32)}, "stencil_cells_index"),
    ({"nt": np.array([1, 3, 1, 1], np.int32)}, "type"),
    ({"nc": np.array([[0, 5], [0, 1], [0, -1], [1, -1]], np.int32)}, "cells_index"),
])
def test_invalid_containers_are_rejected(over, needle):
    rc, msg = _create(_tiny_mesh(**over))
    assert rc == nat_EINVAL() and needle in msg


def test_unknown_scheme_rejected():
    rc, msg = _create(_tiny_mesh(), scheme=7)
    assert rc == nat_EINVAL() and "Unknown flux scheme" in msg


@pytest.mark.parametrize("kernel", [-1, 6, 10, 42])
def test_unknown_kernel_family_rejected(kernel):
    rc, msg = _create(_tiny_mesh(), kernel=kernel)
    assert rc == nat_EINVAL() and "unknown kernel family" in msg


def nat_EINVAL():
    return -1
