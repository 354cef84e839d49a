"""Gradients of the EAM Chebyshev and LJ potentials with respect to their
parameters (energy and force-matching loss) and the trajectory adjoint.

CPU: the oracle's FP64 gradients (oracle/adjoint_oracle.c) against central
finite differences of the oracle's own energies and losses.  GPU: the
library's adjoint kernels against the oracle gradients, against finite
differences of the library's FP64 forward path, and the reverse
velocity-Verlet gradient of the potential energy after 200 steps
(checkpoints every 20) against central finite differences of whole
trajectories (h = 1e-6 relative, tolerance 1e-4 relative)."""
import ctypes as C

import numpy as np
import pytest

import comd_gb300 as cg
from comd_gb300.abi import LjPotential, by_id
from helpers import Case

H_REL = 1e-6


def cheb_base(case):
    ch = case.cheb.contents
    ser = [ch.phi.contents, ch.rho.contents, ch.f.contents]
    c = np.concatenate([np.array(p.values[:p.n]) for p in ser])
    return c, np.array([p.x0 for p in ser]), np.array([p.xn for p in ser])


def step_size(c, k):
    """h = 1e-6 relative to the coefficient (floored at 1e-3 of its series' scale)"""
    q = (k // 32) * 32
    return H_REL * max(abs(c[k]), 1e-3 * np.abs(c[q:q + 32]).max())


def perturbed_target(oracle, case, c, x0, xn, seed=3, rel=0.02):
    """target forces from +-2 % seeded perturbed coefficients (by atom id)"""
    rng = np.random.default_rng(seed)
    oracle.cheb_set(case.cheb, c * (1 + rel * rng.uniform(-1, 1, c.size)), x0, xn)
    case.oracle_force()
    t = by_id(case.o, "f")[:, :3].copy()
    oracle.cheb_set(case.cheb, c, x0, xn)
    return t


def rel_err(g, ref):
    return np.linalg.norm(g - ref) / np.linalg.norm(ref)


# ---------------------------------------------------------------- CPU ----

def test_oracle_eam_gradients_match_finite_differences(oracle):
    case = Case(oracle, cg.POT_EAM_CHEBY, n=(4, 4, 4), amp=0.08, temp=600.0)
    try:
        c, x0, xn = cheb_base(case)
        t = perturbed_target(oracle, case, c, x0, xn)
        U, gu, L, gl = oracle.grad(case.o, "eam", t.reshape(-1))
        fu, fl = np.zeros(96), np.zeros(96)
        for k in range(96):
            h = step_size(c, k)
            vals = []
            for sgn in (1, -1):
                cc = c.copy()
                cc[k] += sgn * h
                oracle.cheb_set(case.cheb, cc, x0, xn)
                case.oracle_force()
                f = by_id(case.o, "f")[:, :3]
                vals.append((case.o.contents.e, ((f - t) ** 2).sum()))
            fu[k] = (vals[0][0] - vals[1][0]) / (2 * h)
            fl[k] = (vals[0][1] - vals[1][1]) / (2 * h)
        oracle.cheb_set(case.cheb, c, x0, xn)
        assert rel_err(gu, fu) < 1e-5
        assert rel_err(gl, fl) < 1e-5
        assert L > 0
    finally:
        case.close()


def test_oracle_lj_gradients_match_finite_differences(oracle):
    case = Case(oracle, cg.POT_LJ, n=(5, 5, 5), amp=0.05, temp=300.0)
    try:
        lp = C.cast(case.o.contents.pot, C.POINTER(LjPotential)).contents
        e0, s0 = lp.epsilon, lp.sigma

        def run(eps, sg, t=None):
            lp.epsilon, lp.sigma = eps, sg
            case.oracle_force()
            f = by_id(case.o, "f")[:, :3].copy()
            return case.o.contents.e, (0.0 if t is None else ((f - t) ** 2).sum()), f

        t = run(e0 * 1.02, s0 * 0.99)[2]
        lp.epsilon, lp.sigma = e0, s0
        U, gu, L, gl = oracle.grad(case.o, "lj", t.reshape(-1))
        for i, (de, ds) in enumerate([(1, 0), (0, 1)]):
            h = H_REL * (e0 if de else s0)
            p = run(e0 + de * h, s0 + ds * h, t)
            m = run(e0 - de * h, s0 - ds * h, t)
            assert abs(gu[i] - (p[0] - m[0]) / (2 * h)) <= 1e-5 * abs(gu[i])
            assert abs(gl[i] - (p[1] - m[1]) / (2 * h)) <= 1e-5 * abs(gl[i])
        lp.epsilon, lp.sigma = e0, s0
    finally:
        case.close()


# ---------------------------------------------------------------- GPU ----

@pytest.mark.gpu
def test_gpu_eam_gradients_match_oracle(oracle):
    case = Case(oracle, cg.POT_EAM_CHEBY, n=(6, 6, 6), amp=0.08, temp=600.0)
    try:
        c, x0, xn = cheb_base(case)
        t = perturbed_target(oracle, case, c, x0, xn)
        U, gu, L, gl = oracle.grad(case.o, "eam", t.reshape(-1))
        d = case.device()
        try:
            Ug, gug = d.energy_grad()
            Lg, glg = d.force_loss_grad(t)
        finally:
            d.close()
        assert abs(Ug - U) <= 1e-12 * abs(U)
        assert abs(Lg - L) <= 1e-9 * L
        assert rel_err(gug, gu) < 1e-11
        assert rel_err(glg, gl) < 1e-9
    finally:
        case.close()


@pytest.mark.gpu
def test_gpu_lj_gradients_match_oracle(oracle):
    case = Case(oracle, cg.POT_LJ, n=(5, 5, 5), amp=0.05, temp=300.0)
    try:
        rng = np.random.default_rng(5)
        case.oracle_force()
        t = by_id(case.o, "f")[:, :3] * (1 + 0.05 * rng.standard_normal((case.o.contents.ntot, 3)))
        U, gu, L, gl = oracle.grad(case.o, "lj", t.reshape(-1))
        d = case.device()
        try:
            Ug, gug = d.energy_grad()
            Lg, glg = d.force_loss_grad(t)
        finally:
            d.close()
        assert abs(Ug - U) <= 1e-12 * abs(U)
        assert np.allclose(gug, gu, rtol=1e-11, atol=0)
        assert abs(Lg - L) <= 1e-10 * L
        assert np.allclose(glg, gl, rtol=1e-9, atol=0)
    finally:
        case.close()


@pytest.mark.gpu
def test_gpu_set_cheby_forces_match_oracle(oracle):
    """coefficients replaced on the device derive the same derivative series
    as the oracle (genDer): FP64 forces agree after the replacement"""
    case = Case(oracle, cg.POT_EAM_CHEBY, n=(6, 6, 6), amp=0.05, temp=300.0)
    try:
        c, x0, xn = cheb_base(case)
        cp = c * (1 + 0.02 * np.random.default_rng(9).uniform(-1, 1, c.size))
        oracle.cheb_set(case.cheb, cp, x0, xn)
        case.oracle_force()
        d = case.device()
        try:
            c_back, a_back, b_back = d.get_cheby()
            d.set_cheby(cp, x0, xn)
            assert np.array_equal(d.get_cheby()[0], cp)
            e = d.force()[0]
            d.download(case.s)
        finally:
            d.close()
        fo = by_id(case.o, "f")[:, :3]
        fg = by_id(case.s, "f")[:, :3]
        assert np.abs(fg - fo).max() <= 1e-10 * np.abs(fo).max()
        assert abs(e - case.o.contents.e) <= 1e-12 * abs(e)
    finally:
        case.close()


@pytest.mark.gpu
def test_gpu_force_loss_gradient_matches_finite_differences(oracle):
    case = Case(oracle, cg.POT_EAM_CHEBY, n=(6, 6, 6), amp=0.08, temp=600.0)
    try:
        c, x0, xn = cheb_base(case)
        t = perturbed_target(oracle, case, c, x0, xn)
        d = case.device()
        try:
            _, g = d.force_loss_grad(t)
            ks = [int(np.argmax(np.abs(g[32 * q:32 * q + 32]))) + 32 * q for q in range(3)]
            ks += list(np.random.default_rng(1).choice(96, 9, replace=False))
            for k in ks:
                h = step_size(c, k)
                vals = []
                for sgn in (1, -1):
                    cc = c.copy()
                    cc[k] += sgn * h
                    d.set_cheby(cc, x0, xn)
                    vals.append(d.force_loss_grad(t)[0])
                fd = (vals[0] - vals[1]) / (2 * h)
                assert abs(g[k] - fd) <= 1e-4 * max(abs(fd), 1e-3 * np.abs(g).max()), k
        finally:
            d.close()
    finally:
        case.close()


def traj_fd(d, case, c, x0, xn, k, n, h):
    vals = []
    for sgn in (1, -1):
        cc = c.copy()
        cc[k] += sgn * h
        d.set_cheby(cc, x0, xn)
        d.upload(case.s)
        vals.append(d.steps(n, 1e-15)[0])
    return (vals[0] - vals[1]) / (2 * h)


@pytest.mark.gpu
@pytest.mark.parametrize("n,every,tol", [(40, 8, 1e-6), (200, 20, 1e-4)])
def test_gpu_trajectory_adjoint_matches_finite_differences(oracle, n, every, tol):
    """dJ/dc for J = potential energy after n velocity-Verlet steps (1 fs,
    checkpoints every `every`) against central differences of whole
    trajectories, h = 1e-6 relative.  J is only piecewise smooth in c: the
    Chebyshev phi and rho do not vanish at the cutoff, so a pair crossing it
    at some step adds a jump.  A difference bracket that holds such a jump is
    recognised by repeating it with h/4 (the two disagree) and not used; the
    test needs at least 6 usable components."""
    case = Case(oracle, cg.POT_EAM_CHEBY, n=(5, 5, 5), amp=0.05, temp=600.0)
    try:
        c, x0, xn = cheb_base(case)
        d = cg.DeviceSim(case.s, cg.opts(cg.POT_EAM_CHEBY, cg.PREC_FP64, True,
                                         cheby_from_host=True, per_step_lists=True))
        try:
            j, g = d.traj_energy_grad(n, 1e-15, every)
            ks = [int(np.argmax(np.abs(g[32 * q:32 * q + 32]))) + 32 * q for q in range(3)]
            ks += [1, 5, 8, 33, 40, 66, 70]
            used = 0
            for k in ks:
                h = step_size(c, k)
                fd = traj_fd(d, case, c, x0, xn, k, n, h)
                fd4 = traj_fd(d, case, c, x0, xn, k, n, h / 4)
                scale = max(abs(fd), 1e-3 * np.abs(g).max())
                if abs(fd - fd4) > 1e-6 * scale:
                    continue  # a cutoff crossing inside the bracket
                used += 1
                assert abs(g[k] - fd) <= tol * scale, (k, g[k], fd, fd4)
            assert used >= 6
            # J is the energy the forward loop reaches
            d.set_cheby(c, x0, xn)
            d.upload(case.s)
            assert abs(d.steps(n, 1e-15)[0] - j) <= 1e-9 * abs(j)
        finally:
            d.close()
    finally:
        case.close()
