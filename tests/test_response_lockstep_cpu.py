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
