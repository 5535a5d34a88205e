"""Shared case builders for the GPU parity tests: the same inputs for the CUDA path (via the
package) and for the oracle."""
import numpy as np

QUADS = ["D2Q4", "D2Q5", "D2Q9", "D2Q13", "D2Q17", "D2Q21", "D2Q37"]


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    nz = b != 0
    zero_ok = np.all(a[~nz] == 0) if np.any(~nz) else True
    e = float(np.max(np.abs(a[nz] - b[nz]) / np.abs(b[nz]))) if np.any(nz) else 0.0
    return e if zero_ok else float("inf")


def wave_field(q, nx, ny, seed=0, amp=0.02):
    """A smooth non-equilibrium start: Hermite equilibrium of a random two-mode velocity field
    plus a small random perturbation, populations (Q, ny, nx)."""
    rng = np.random.default_rng(seed)
    X, Y = np.meshgrid(np.arange(nx), np.arange(ny))
    kx, ky = 2 * np.pi / max(nx, 1), 2 * np.pi / max(ny, 1)
    a = rng.normal(size=4)
    ux = amp * (a[0] * np.sin(ky * Y + 0.3) + a[1] * np.cos(kx * X))
    uy = amp * (a[2] * np.sin(kx * X + 0.7) + a[3] * np.cos(ky * Y))
    rho = 1.0 + 0.01 * np.cos(kx * X + ky * Y)
    from oracle import oracle as O
    f = np.empty((len(q.weights), ny, nx))
    for y in range(ny):
        for x in range(nx):
            f[:, y, x] = O.hermite_equilibrium(q.name, rho[y, x], (ux[y, x], uy[y, x]), 1.0)
    f *= 1.0 + 1e-3 * rng.normal(size=f.shape)
    return f
