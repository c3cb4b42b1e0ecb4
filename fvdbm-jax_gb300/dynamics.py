"""D2Q9 and D2Q13 lattices (reference ``src/dynamics.py:50-102``) and the
float32 scalars the kernels need.

The reference keeps every array in float32 (x64 is never enabled) and treats
``tau``/``delta_t`` as Python scalars, so:

* ``C = 1/sqrt(3)`` is a float32 (``src/dynamics.py:64``); ``C**2`` and
  ``C**4`` are float32 repeated squarings; the kernels receive ``c2 = C*C``,
  ``c4x2 = 2*((C*C)*(C*C))`` and ``c2x2 = 2*(C*C)``;
* ``1 / tau`` is evaluated in Python double and then rounded to float32 when
  it multiplies a float32 array (``src/containers.py:121``), hence
  ``inv_tau = float32(1/tau)``;
* ``delta_t`` enters float32 arithmetic as ``float32(delta_t)``.
"""
from __future__ import annotations

import numpy as np

F32 = np.float32


class D2Q9:
    """D2Q9 dynamics with relaxation time ``tau`` and time step ``delta_t``
    (reference ``D2Q9(tau, delta_t)``, ``src/dynamics.py:65-68``)."""

    DIM = 2
    NUM_QUIVERS = 9
    KSI = np.array([[0, 0], [1, 0], [0, 1], [-1, 0], [0, -1],
                    [1, 1], [-1, 1], [-1, -1], [1, -1]], dtype=np.int32)
    W = np.array([4 / 9, 1 / 9, 1 / 9, 1 / 9, 1 / 9, 1 / 36, 1 / 36, 1 / 36, 1 / 36], dtype=F32)
    C = F32(1) / np.sqrt(F32(3))

    def __init__(self, tau, delta_t):
        self.tau = tau
        self.delta_t = delta_t

    # float32 constants exactly as the reference's expressions produce them
    @property
    def c2(self) -> np.float32:
        return F32(self.C * self.C)

    @property
    def c4x2(self) -> np.float32:
        c2 = F32(self.C * self.C)
        return F32(F32(2) * F32(c2 * c2))

    @property
    def c2x2(self) -> np.float32:
        return F32(F32(2) * F32(self.C * self.C))

    c6x2 = F32(0)  # (third-order term of D2Q13 only)

    @property
    def inv_tau(self) -> np.float32:
        return F32(np.asarray(1 / self.tau).astype(F32))

    @property
    def dt32(self) -> np.float32:
        return F32(np.asarray(self.delta_t).astype(F32))

    def calc_eq(self, rho, vel) -> np.ndarray:
        """Second-order BGK equilibrium (``src/dynamics.py:70-74``) for
        ``rho`` [..., 1] and ``vel`` [..., 2], in the reference's float32
        operation order: ``(W*rho) * (((1 + a/c2) + a*a/c4x2) - u.u/c2x2)``
        with ``a = xi.u`` folded over x then y."""
        rho = np.asarray(rho, dtype=F32)
        vel = np.asarray(vel, dtype=F32)
        ksi = self.KSI.astype(F32)
        a = ksi[:, 0] * vel[..., 0:1] + ksi[:, 1] * vel[..., 1:2]
        uu = vel[..., 0:1] * vel[..., 0:1] + vel[..., 1:2] * vel[..., 1:2]
        inner = ((F32(1) + a / self.c2) + (a * a) / self.c4x2) - uu / self.c2x2
        return (self.W * rho) * inner

    def rest_pdf(self) -> np.ndarray:
        """feq(rho=1, u=0): the default pdf of every container element
        (``src/containers.py:29``).  Equal to W."""
        return self.W.copy()

    def __repr__(self) -> str:
        return f"D2Q9(tau={self.tau}, delta_t={self.delta_t})"


class D2Q13(D2Q9):
    """D2Q13 dynamics (reference ``D2Q13(tau, delta_t)``,
    ``src/dynamics.py:77-102``): 13 velocities including (+-2, 0), (0, +-2),
    C = 1/sqrt(2) in float32, and the third-order equilibrium
    ``(W*rho) * ((((1 + a/C^2) + a^2/(2C^4)) - u.u/(2C^2)) + a^3/(2C^6) - 3 a u.u/(2C^4))``
    with the powers of C and a formed as jax's integer_pow forms them
    (C^4 = (C*C)*(C*C), C^6 = (C*C)*C^4, a^3 = a*(a*a))."""

    NUM_QUIVERS = 13
    KSI = np.array([[0, 0], [1, 0], [0, 1], [-1, 0], [0, -1], [1, 1], [-1, 1], [-1, -1], [1, -1],
                    [2, 0], [0, 2], [-2, 0], [0, -2]], dtype=np.int32)
    W = np.array([3 / 8, 1 / 12, 1 / 12, 1 / 12, 1 / 12, 1 / 16, 1 / 16, 1 / 16, 1 / 16,
                  1 / 96, 1 / 96, 1 / 96, 1 / 96], dtype=F32)
    C = F32(1) / np.sqrt(F32(2))

    @property
    def c6x2(self) -> np.float32:
        c2 = F32(self.C * self.C)
        return F32(F32(2) * F32(c2 * F32(c2 * c2)))

    def calc_eq(self, rho, vel) -> np.ndarray:
        rho = np.asarray(rho, dtype=F32)
        vel = np.asarray(vel, dtype=F32)
        ksi = self.KSI.astype(F32)
        a = ksi[:, 0] * vel[..., 0:1] + ksi[:, 1] * vel[..., 1:2]
        uu = vel[..., 0:1] * vel[..., 0:1] + vel[..., 1:2] * vel[..., 1:2]
        inner = ((((F32(1) + a / self.c2) + (a * a) / self.c4x2) - uu / self.c2x2)
                 + (a * (a * a)) / self.c6x2) - ((F32(3) * a) * uu) / self.c4x2
        return (self.W * rho) * inner

    def __repr__(self) -> str:
        return f"D2Q13(tau={self.tau}, delta_t={self.delta_t})"


def as_lattice(dyn):
    """This package's dynamics object for any dynamics with tau/delta_t
    (the reference's D2Q9/D2Q13 or these), chosen by NUM_QUIVERS."""
    if isinstance(dyn, D2Q9):
        return dyn
    cls = D2Q13 if int(getattr(dyn, "NUM_QUIVERS", 9)) == 13 else D2Q9
    return cls(dyn.tau, dyn.delta_t)
