"""The lockstep response driver (response.solve_responses) is host logic: its DIIS
bookkeeping (history truncation before the append, Gram rows, bordered solve), the
energy-derivative update and the per-response convergence test.  Here it runs on CPU
tensors against a small dense stand-in for the CISD plan (same method names and
meanings: residual with RES_CONST / RES_ETERM flags, Jacobi update by 1/D, weighted
Gram rows, the fused combination with its energy), and each response solved in lockstep
must follow exactly the iterations it follows alone."""
import numpy as np
import torch

from apyib_gb300 import _lib
from apyib_gb300.response import solve_response, solve_responses


class DensePlan:
    """r(t) = [c] + L t [- E t], update t + r / D, energy sum t * ew; singles are the first n1."""

    def __init__(self, L, c, ew, D, n1):
        self.L, self.c, self.ew, self.D = L, c, ew, D
        self.n1, self.n2 = n1, L.shape[0] - n1
        self.o, self.v, self.singles, self.mixed = 2, 3, True, False

    def vec(self):
        return torch.empty(self.n1 + self.n2, dtype=torch.complex128)

    def residual(self, t, E, precision=0, flags=_lib.RES_CONST | _lib.RES_ETERM, out=None):
        r = self.L @ t
        if flags & _lib.RES_CONST:
            r = r + self.c
        if flags & _lib.RES_ETERM:
            r = r - complex(E) * t
        return r

    def update(self, t, r, out=None):
        return t + r / self.D

    def dots_into(self, x, ys, out):
        w = torch.ones(self.n1 + self.n2, dtype=torch.float64)
        w[self.n1:] = 4.0
        for j, y in enumerate(ys):
            out[j] = torch.sum(w * y.conj() * x)
        return out

    def dots(self, x, ys):
        out = torch.empty(16, dtype=torch.complex128)
        return self.dots_into(x, ys, out)[:len(ys)].numpy().copy()

    def combine_into(self, ys, coefs, t_old, t_new, out3):
        s = sum(complex(c) * y for c, y in zip(coefs, ys))
        t_new.copy_(s)
        out3[0] = torch.sum(s * self.ew)
        return out3

    def combine(self, ys, coefs, t_old, t_new):
        out = torch.empty(3, dtype=torch.complex128)
        self.combine_into(ys, coefs, t_old, t_new, out)
        return complex(out[0]), 0j, 0j

    def lincomb(self, ys, coefs, out=None):
        return sum(complex(c) * y for c, y in zip(coefs, ys))


def _problem(rng, n=24, n1=6):
    D = torch.as_tensor(-(1.0 + rng.random(n)) * 2.0)
    # the residual carries the Fock diagonal, -D t, so that the Jacobi step t + r / D contracts
    L = torch.diag(-D).to(torch.complex128) + torch.as_tensor(
        0.05 * (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))))
    c = torch.as_tensor(rng.standard_normal(n) + 1j * rng.standard_normal(n))
    ew = torch.as_tensor(0.1 * (rng.standard_normal(n) + 1j * rng.standard_normal(n)))
    return L, c, ew, D, n1


def test_lockstep_equals_one_at_a_time_on_cpu():
    rng = np.random.default_rng(5)
    L, c, ew, D, n1 = _problem(rng)
    plan = DensePlan(L, c, ew, D, n1)
    t = torch.as_tensor(0.1 * (rng.standard_normal(L.shape[0]) + 1j * rng.standard_normal(L.shape[0])))
    E = complex(torch.sum(t * ew))
    pxs = []
    n = L.shape[0]
    for s in (0.01, 0.3, 2.0):                # perturbations of different size converge at different steps
        # a perturbation enters only through c^x + L^x t and the energy weights EW^x
        Lx = torch.as_tensor(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
        cx = torch.as_tensor(rng.standard_normal(n) + 1j * rng.standard_normal(n))
        ewx = torch.as_tensor(rng.standard_normal(n) + 1j * rng.standard_normal(n))
        pxs.append(DensePlan(s * Lx, s * cx, s * ewx, D, n1))
    for diis in (True, False):
        params = dict(e_convergence=1e-12, d_convergence=1e-11, max_iterations=200, DIIS=diis)
        hist = [[] for _ in pxs]
        together = solve_responses(plan, pxs, t, E, params, histories=hist)
        lengths = {len(h) for h in hist}
        if diis:
            assert len(lengths) > 1                # the responses did stop at different iterations
        for k, px in enumerate(pxs):
            h1 = []
            dE, dt = solve_response(plan, px, t, E, params, history=h1)
            assert len(h1) == len(hist[k]) < 200
            assert together[k][0] == dE
            assert torch.equal(together[k][1], dt)
            # converged: the response equation holds, r^x = c^x + L^x t + (L - E) t^x - E^x t = 0
            rx = px.residual(t, 0.0, flags=_lib.RES_CONST) + plan.residual(dt, E, flags=_lib.RES_ETERM) - dE * t
            assert torch.abs(rx).max().item() < 1e-9


def test_imaginary_response_needs_the_conjugated_step_norm():
    """A magnetic-field perturbation of a real problem gives purely imaginary t^x.  The
    reference sums the unconjugated squares of the step (apyib/analytic_aats.py:868-879),
    in its real formulation of the magnetic responses; applied to imaginary t^x that sum is
    negative, its square root imaginary, and numpy's complex < real compares the real part,
    0, so the step test would pass at every iteration.  The driver uses conjugated squares:
    it stops only once the step is small, and the response it returns solves its equation."""
    rng = np.random.default_rng(9)
    n, n1 = 24, 6
    D = torch.as_tensor(-(1.0 + rng.random(n)) * 2.0)
    L = torch.diag(-D).to(torch.complex128) + torch.as_tensor(0.05 * rng.standard_normal((n, n)) + 0j)
    c = torch.as_tensor(rng.standard_normal(n) + 0j)
    ew = torch.as_tensor(0.1 * rng.standard_normal(n) + 0j)
    plan = DensePlan(L, c, ew, D, n1)
    t = torch.as_tensor(0.1 * rng.standard_normal(n) + 0j)
    E = complex(torch.sum(t * ew))
    # purely imaginary perturbation (i times real matrices), as the magnetic field's -i L / 2
    px = DensePlan(torch.as_tensor(1j * rng.standard_normal((n, n))), torch.as_tensor(1j * rng.standard_normal(n)),
                   torch.as_tensor(1j * rng.standard_normal(n)), D, n1)
    d_conv = 1e-10
    params = dict(e_convergence=1e-12, d_convergence=d_conv, max_iterations=200, DIIS=True)
    hist = []
    dE, dt = solve_response(plan, px, t, E, params, history=hist)
    assert torch.abs(dt.real).max().item() < 1e-12 < torch.abs(dt.imag).max().item()
    # the reference's step test, on the unconjugated sums, is vacuous from the first iteration on
    for h in hist:
        assert np.complex128(h["rms_t2_unconj"]) < d_conv and np.complex128(h["rms_t1_unconj"]) < d_conv
    # at iteration 2 the step is still far from converged
    assert abs(hist[1]["rms_t2"]) > 1e3 * d_conv
    # the driver's conjugated step norm is what ends the iteration, and the response solves its equation
    assert len(hist) > 2 and abs(hist[-1]["rms_t2"]) < d_conv and abs(hist[-1]["rms_t1"]) < d_conv
    rx = px.residual(t, 0.0, flags=_lib.RES_CONST) + plan.residual(dt, E, flags=_lib.RES_ETERM) - dE * t
    assert torch.abs(rx).max().item() < 1e-9
