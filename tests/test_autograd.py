"""The parameter derivatives behind a torch.autograd.Function (test harness only).

``NonbondedEnergy`` maps (charges per atom, eps per LJ type, sigma per LJ type) to E_total
through ``moil_nb_adjoint`` -- one evaluation (the PME grid recomputed, not stored) plus the
adjoint kernels -- and returns dE/dq per atom and dE/deps, dE/dsigma per type (the per-atom
derivatives summed over each type's atoms) from ``backward``.  MOIL differentiates with respect
to no parameter, so the checks are independent derivatives of the same energy:

* central finite differences (h = 1e-4 relative) of the plain FP64 GPU energy, which is exact
  to about 1e-12: the FP64 handle's gradient to 1e-6, the mixed handle's to 1e-4;
* the oracle's FP64 adjoint (ora_adjoint_mi) per type and per atom: the mixed handle's per-type
  derivatives to 1e-4 relative, its charge derivatives to 1e-5 relative RMS;

on four of the 64 perturbed copies of the 23,558-atom solute system (eps, sigma per LJ type and
the solute charges each perturbed by up to 1%).  Charge directions perturb solute atoms only and
sum to zero (systems stay neutral, waters keep identical charges).
"""
import numpy as np
import pytest

from conftest import rel_rms
from moil_fnrfd_gb300 import systems as S
from moil_fnrfd_gb300.nb import MOIL_NB_FP64, MOIL_NB_MIXED, Nonbonded
from oracle import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

H = 1e-4
COPIES = (0, 21, 42, 63)


def lj_types(s):
    """Each atom's LJ type: the distinct (eps, sigma) pairs, as the perturbed copies use them."""
    eps, sig = S.lj_decode(s)
    types, tid = np.unique(np.round(np.stack([eps, sig], axis=1), 12), axis=0, return_inverse=True)
    tid = tid.reshape(-1)
    eps_t = np.array([eps[tid == k][0] for k in range(len(types))])
    sig_t = np.array([sig[tid == k][0] for k in range(len(types))])
    return tid, eps_t, sig_t


def make_system(base, q, eps_t, sig_t, tid):
    s = base.copy()
    s.ptchg = np.array(q, dtype=np.float64)
    return S.with_lj(s, np.asarray(eps_t)[tid], np.asarray(sig_t)[tid])   # 1-4 parameters re-derived


class NonbondedEnergy(torch.autograd.Function):
    """E_total(q, eps_type, sigma_type) of one system; backward from moil_nb_adjoint."""

    @staticmethod
    def forward(ctx, q, eps_t, sig_t, base, tid, precision):
        s = make_system(base, q.detach().numpy(), eps_t.detach().numpy(), sig_t.detach().numpy(), tid)
        nb = Nonbonded(s, precision=precision)
        dq, de, ds = nb.adjoint(s.coor)
        e = nb.energies()[0]["e_total"]
        nb.close()
        n = eps_t.numel()
        ctx.save_for_backward(torch.from_numpy(dq), torch.from_numpy(np.bincount(tid, de, n)),
                              torch.from_numpy(np.bincount(tid, ds, n)))
        return torch.tensor(e, dtype=torch.float64)

    @staticmethod
    def backward(ctx, g):
        dq, de, ds = ctx.saved_tensors
        return g * dq, g * de, g * ds, None, None, None


def gpu_energy(base, q, eps_t, sig_t, tid, precision=MOIL_NB_FP64):
    s = make_system(base, q, eps_t, sig_t, tid)
    nb = Nonbonded(s, precision=precision)
    _, e = nb.eforce(s.coor)
    nb.close()
    return e["e_total"]


@pytest.fixture(scope="module")
def copies(cfg1):
    return S.perturbed_copies(cfg1, 64)


def grads(base, precision):
    tid, eps_t, sig_t = lj_types(base)
    q = torch.tensor(base.ptchg, dtype=torch.float64, requires_grad=True)
    e_t = torch.tensor(eps_t, requires_grad=True)
    s_t = torch.tensor(sig_t, requires_grad=True)
    E = NonbondedEnergy.apply(q, e_t, s_t, base, tid, precision)
    E.backward()
    return tid, eps_t, sig_t, q.grad.numpy(), e_t.grad.numpy(), s_t.grad.numpy(), float(E.detach())


def solute_direction(base, seed):
    """A random charge direction over the solute atoms with zero sum."""
    solute = np.zeros(base.npt, dtype=bool)
    first = 0
    for m in range(base.totmon):
        last = int(base.poipt[m])
        if base.montype[m] == S.MON_OTHER:
            solute[first:last] = True
        first = last
    v = np.zeros(base.npt)
    v[solute] = np.random.default_rng(seed).standard_normal(int(solute.sum()))
    v[solute] -= v[solute].mean()
    return v / np.linalg.norm(v)


@pytest.mark.parametrize("precision", [MOIL_NB_FP64, MOIL_NB_MIXED], ids=["fp64", "mixed"])
def test_autograd_against_fp64_finite_differences(copies, precision):
    base = copies[0]
    tid, eps_t, sig_t, gq, ge, gs, _ = grads(base, precision)
    tol = 1e-6 if precision == MOIL_NB_FP64 else 1e-4
    q0 = base.ptchg
    for k in range(len(eps_t)):
        if eps_t[k] <= 0.0:
            continue                      # LJ-free atoms (hydrogens): no LJ parameter to move
        for vec, base_t, got in ((0, eps_t, ge), (1, sig_t, gs)):
            h = H * base_t[k]

            def at(d):
                e, g = eps_t.copy(), sig_t.copy()
                (e if vec == 0 else g)[k] += d
                return gpu_energy(base, q0, e, g, tid)
            fd = (at(+h) - at(-h)) / (2.0 * h)
            print(f"type {k} {'eps' if vec == 0 else 'sigma'}: autograd {got[k]:.8e} fd {fd:.8e}")
            # types with a small share of the energy are held to the same tolerance on the
            # scale of the largest per-type derivative
            assert got[k] == pytest.approx(fd, rel=tol, abs=1e-2 * tol * np.abs(got).max()), (k, vec)
    for seed in (1, 2):
        v = solute_direction(base, seed)
        h = H * float(np.sqrt((q0[v != 0] ** 2).mean()))
        fd = (gpu_energy(base, q0 + h * v, eps_t, sig_t, tid) - gpu_energy(base, q0 - h * v, eps_t, sig_t, tid)) / (2 * h)
        print(f"charge direction {seed}: autograd {gq @ v:.8e} fd {fd:.8e}")
        assert gq @ v == pytest.approx(fd, rel=tol)


@pytest.mark.parametrize("k", COPIES)
def test_autograd_mixed_against_the_oracle_adjoint(copies, k):
    base = copies[k]
    tid, eps_t, sig_t, gq, ge, gs, _ = grads(base, MOIL_NB_MIXED)
    dq, de, ds = O.adjoint(base)
    n = len(eps_t)
    we, ws = np.bincount(tid, de, n), np.bincount(tid, ds, n)
    assert rel_rms(gq, dq) < 1e-5
    for t in range(n):
        if eps_t[t] <= 0.0:
            continue
        assert ge[t] == pytest.approx(we[t], rel=1e-4, abs=1e-6 * np.abs(we).max()), ("eps", t)
        assert gs[t] == pytest.approx(ws[t], rel=1e-4, abs=1e-6 * np.abs(ws).max()), ("sigma", t)
