"""Host-side mirror of the reference API (no GPU): quadratures, kinetics, problems, initial
conditions, collision-model factories and the processing-event logic, against the oracle;
and the C ABI library's exported symbols against include/lbm_gb300.h."""
import ctypes
import math
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
QUADS = ["D2Q4", "D2Q5", "D2Q9", "D2Q13", "D2Q17", "D2Q21", "D2Q37"]


def _rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    scale = np.maximum(np.abs(b), 1e-300)
    return float(np.max(np.where(b == 0, np.abs(a), np.abs(a - b) / scale)))


@pytest.mark.parametrize("qname", QUADS)
def test_quadrature_tables_bitwise(lbm, O, qname):
    q = lbm.Quadratures[qname]
    ref = O.quadrature(qname)
    assert q.Q == ref["Q"] and lbm.order(q) == ref["order"]
    assert q.speed_of_sound_squared == ref["cs"]
    assert np.array_equal(q.weights, ref["w"])
    assert np.array_equal(q.abscissae[0], ref["cx"]) and np.array_equal(q.abscissae[1], ref["cy"])
    assert np.array_equal(q.opposites, ref["opposite"])
    for i in range(q.Q):
        assert lbm.opposite(q, i + 1) == ref["opposite"][i] + 1


@pytest.mark.parametrize("qname", QUADS)
def test_kinetics_against_oracle(lbm, O, qname):
    q = lbm.Quadratures[qname]
    for rho, u, T in [(1.0, (0.01, -0.02), 1.0), (1.03, (0.1, 0.05), 1.0), (0.98, (0.0, 0.03), 1.02)]:
        assert _rel(lbm.equilibrium(q, rho, u, T), O.hermite_equilibrium(qname, rho, u, T)) <= 1e-15
        assert _rel(lbm.equilibrium_(q, rho, u), O.equilibrium(qname, rho, u)) <= 1e-15
        f = O.hermite_equilibrium(qname, rho, u, T) * (1 + 1e-3 * np.arange(q.Q) / q.Q)
        m = O.moments(qname, f, 0.8)
        assert lbm.density(q, f) == pytest.approx(m[0], rel=1e-15)
        ux, uy = lbm.velocity(q, f)
        assert ux == pytest.approx(m[1], rel=1e-14) and uy == pytest.approx(m[2], rel=1e-14)
        assert lbm.pressure(q, f) == pytest.approx(m[3], rel=1e-14)
        s = lbm.deviatoric_tensor(q, 0.8, f)
        np.testing.assert_allclose([s[0, 0], s[1, 0], s[0, 1], s[1, 1]], m[5:9], rtol=1e-12, atol=1e-17)


class InitializationTestProblem:
    """test/initial_conditions.jl:12-87, as a user subclass of FluidFlowProblem."""

    @staticmethod
    def make(lbm, N=4, nu=1.0 / 6.0):
        class P(lbm.FluidFlowProblem):
            U = 0.001

            def __init__(self):
                self.u_max, self.ν, self.NX, self.NY, self.domain_size = 1.0, nu, N, N, (1.0, 1.0)

            def pressure(self, q, x, y, t=0.0):
                return 1.0 - (1 / 4) * q.speed_of_sound_squared * self.u_max ** 2 * self.U ** 2 * (
                    np.cos(2 * x) + np.cos(2 * y))

            def density(self, q, x, y, t=0.0):
                return self.pressure(q, x, y, t)

            def velocity(self, x, y, t=0.0):
                s = self.u_max * self.U
                return s * (np.cos(2 * math.pi * x) * np.sin(2 * math.pi * y)), \
                    s * (-np.sin(2 * math.pi * x) * np.cos(2 * math.pi * y))

            def velocity_gradient(self, x, y, t=0.0):
                ux = -np.sin(2 * math.pi * x) * np.sin(2 * math.pi * y)
                vy = np.sin(2 * math.pi * x) * np.sin(2 * math.pi * y)
                uy = np.cos(2 * math.pi * x) * np.cos(2 * math.pi * y)
                vx = -np.cos(2 * math.pi * x) * np.cos(2 * math.pi * y)
                s = self.u_max * self.U * 2 * math.pi
                return np.array([[s * ux, s * vx], [s * uy, s * vy]])

            def deviatoric_tensor(self, q, x, y, t=0.0):
                return super().deviatoric_tensor(q, x, y, t) * self.NX

        return P()


def _problems(lbm, O):
    import math as m
    q9 = lbm.D2Q9()
    yield "tgv_static", lbm.TaylorGreenVortex(0.1, 1, 12, 10), O.taylor_green_vortex(0.1, 1, 12, 10)
    yield "tgv_decay", lbm.TaylorGreenVortex(0.1, 1, 16, 16, static=False), \
        O.taylor_green_vortex(0.1, 1, 16, 16, static=False)
    yield "TGV", lbm.TGV(q9, 0.8, 1, 14, 9, 0.03), O.tgv("D2Q9", 0.8, 1, 14, 9, 0.03)
    yield "poiseuille", lbm.PoiseuilleFlow(0.1, 2), O.poiseuille(0.1, 2)
    yield "couette", lbm.CouetteFlow(1 / 6, 2), O.couette(1 / 6, 2)
    yield "shear_static", lbm.DecayingShearFlow(0.1, 2, static=True, k_y=1.0), \
        O.decaying_shear_flow(0.1, 2, static=True, k_y=1.0)
    yield "shear_decay", lbm.DecayingShearFlow(0.1, 2, static=False, A=3.0), \
        O.decaying_shear_flow(0.1, 2, static=False, A=3.0)
    yield "cavity", lbm.LidDrivenCavityFlow(1 / 6, 1, 9, 7), O.lid_driven_cavity(1 / 6, 1, 9, 7)
    yield "init_test", InitializationTestProblem.make(lbm, 8, 1 / 3), O.init_test_problem(8, 1 / 3)
    yield "shear_wave", lbm.ShearWave(12, 12, 0.05), O.shear_wave(12, 12, 0.05)


STRATS = {"zero": 0, "eq": 1, "eq_offeq": 2, "const_density": 3, "velocity_stress": 4}


@pytest.mark.parametrize("qname", ["D2Q9", "D2Q13", "D2Q17", "D2Q37"])
def test_problems_and_initial_conditions(lbm, O, qname):
    q = lbm.Quadratures[qname]
    cls = {"zero": lbm.ZeroVelocityInitialCondition, "eq": lbm.AnalyticalEquilibrium,
           "eq_offeq": lbm.AnalyticalEquilibriumAndOffEquilibrium, "const_density": lbm.ConstantDensity,
           "velocity_stress": lbm.AnalyticalVelocityAndStress}
    for name, P, op in _problems(lbm, O):
        if name == "TGV":
            P = lbm.TGV(q, 0.8, 1, 14, 9, 0.03)
            op = O.tgv(qname, 0.8, 1, 14, 9, 0.03)
        sc = O.problem_scalars(op)
        assert P.delta_x() == sc["delta_x"] and P.delta_t() == sc["delta_t"], name
        assert P.viscosity() == pytest.approx(sc["viscosity"], rel=1e-15), name
        xr, yr, xs, ys = lbm.problem_range(P)
        oxr, oyr = O.problem_coords(op)
        assert np.array_equal(xr, oxr) and np.array_equal(yr, oyr), name
        assert xs == sc["x_step"] and ys == sc["y_step"], name
        for t in (0.0, 0.37):
            F = lbm.analytic_fields(q, P, t)
            R = O.problem_fields(op, qname, t)
            for k, key in enumerate(["rho", "ux", "uy", "p", "sxx", "syx", "sxy", "syy"]):
                assert _rel(F[key], R[k]) <= 1e-13, (name, key, t)
        if P.has_external_force():
            assert _rel(lbm.lattice_force_field(P, 0.2), O.force_field(op, 0.2)) <= 1e-14, name
        for sname, sid in STRATS.items():
            f = lbm.initialize(cls[sname](), q, P)
            assert f.shape == (q.Q, P.NY, P.NX)
            assert _rel(f, O.initialize(sid, qname, op)) <= 1e-14, (name, sname)


def test_collision_model_constructors(lbm):
    q = lbm.D2Q9()
    t = lbm.TRT(0.7, 1.2)  # TRT(τ_a, τ_s): trt.jl:6
    assert t.τ_symmetric == 1.2 and t.τ_asymmetric == 0.7
    p = lbm.PoiseuilleFlow(0.1, 1)
    m = lbm.make_collision_model(lbm.TRT, q, p)
    tau = 3 * 0.1 + 0.5
    assert m.τ_symmetric == tau and m.τ_asymmetric == 0.5 + 0.25 / (tau - 0.5) and m.force == "problem"
    m = lbm.make_collision_model(lbm.TRT_Λ(3 / 16), q, p)
    assert m.τ_asymmetric == 0.5 + (3 / 16) / (tau - 0.5)
    assert lbm.MRT(q, 0.8).τs == [0.8, 0.8]                    # round(Int, 5/2) = 2
    assert lbm.MRT(lbm.D2Q17(), 0.8).τs == [0.8] * 4           # round(Int, 7/2) = 4
    assert lbm.MRT(lbm.D2Q37(), 0.6, 0.9).τs == [0.6, 0.9, 0.6, 0.9]
    assert lbm.MRT(q, 0.8, "problem").force is None             # the reference drops it
    assert lbm.MRT(q, [0.8, 0.9], force="problem").force == "problem"
    s = lbm.make_collision_model(lbm.SRT, q, lbm.TaylorGreenVortex(0.1, 1, static=False))
    assert s.τ == tau and s.force is None


def test_processing_events(lbm):
    p = lbm.PoiseuilleFlow(0.1, 1)
    pm = lbm.TrackHydrodynamicErrors(p, False, 5000, lbm.VelocityConvergenceStoppingCriteria(1e-7, p))
    assert pm.next_event(1) == 100 and pm.next_event(101) == 200 and pm.next_event(4950) == 5000
    pm = lbm.TrackHydrodynamicErrors(lbm.TaylorGreenVortex(0.1, 1, static=False), False, 1000)
    assert pm.next_event(1) == 1000 and pm.next_event(1001) is None
    pm = lbm.TrackHydrodynamicErrors(lbm.TaylorGreenVortex(0.1, 1, static=False), True, 1000)
    assert pm.next_event(7) == 7
    snaps = lbm.TakeSnapshots(p, [5, 17])
    assert snaps.next_event(1) == 5 and snaps.next_event(6) == 17 and snaps.next_event(18) is None
    assert isinstance(lbm.ProcessingMethod(lbm.TGV(lbm.D2Q9(), 0.8), False, 10), lbm.TrackHydrodynamicErrors)
    assert isinstance(lbm.ProcessingMethod(p, False, 10), lbm.CompareWithAnalyticalSolution)
    assert isinstance(lbm.StopCriteria(p), lbm.MeanVelocityStoppingCriteria)


def test_abi_library_exports_every_header_symbol(lbm):
    """The C ABI library loads and exports every function include/lbm_gb300.h declares (no
    device call is made)."""
    header = open(os.path.join(ROOT, "include", "lbm_gb300.h")).read()
    body = re.sub(r"/\*.*?\*/", "", header, flags=re.S)
    names = sorted(set(re.findall(r"\b(lbm_[a-z_0-9]+)\s*\(", body)))
    assert len(names) >= 18
    lbm.build()
    L = ctypes.CDLL(lbm.library_path())
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert set(lbm._native.EXPORTED_SYMBOLS) <= set(names)
    assert L.lbm_abi_version() == 1


def test_product_has_no_cpu_fallback(lbm, monkeypatch):
    """Without the CUDA library the product raises instead of computing on the host."""
    monkeypatch.setattr(lbm._native, "_lib", None)
    monkeypatch.setattr(lbm._native, "library_path", lambda: "/nonexistent/liblbm_gb300.so")
    with pytest.raises(RuntimeError):
        lbm._native.lib()
