"""Mixed-precision ε⁻¹ (FP32 Gauss–Jordan + FP64 refinement with the residual
on the tensor cores) against numpy's FP64 inverse of the same matrices.

The input is what calc_eps holds before its ε block (pygw.py:3229): a
Hermitian χ0-like part P; the library forms A = (P + Pᴴ)/2 + I, inverts it and
returns A⁻¹ − I.  Matrices are I + B·Bᴴ with a chosen spread of eigenvalues
(condition numbers up to ~1e3), sizes that are and are not multiples of the
128/256 tile edges, and frequency batches smaller than the frequency count.
"""
import numpy as np
import pytest
import torch

from pygw_gb300 import eps as peps

pytestmark = pytest.mark.gpu


def _problem(N, nom, cond, seed=0):
    rng = np.random.default_rng(seed)
    P = np.empty((nom, N, N), dtype=np.complex128)
    for w in range(nom):
        q, _ = np.linalg.qr(rng.normal(size=(N, N)) + 1j * rng.normal(size=(N, N)))
        lam = np.exp(np.linspace(0.0, np.log(cond), N))[rng.permutation(N)] - 1.0   # A = I + P: eigenvalues 1..cond
        P[w] = (q * lam) @ q.conj().T
    return P


def _inverse_minus_one(P):
    N = P.shape[1]
    A = (P + np.conj(P.transpose(0, 2, 1))) / 2 + np.eye(N)
    return np.linalg.inv(A) - np.eye(N)


def _run(P, precision, iters=None, omega_batch=None):
    nom, N, _ = P.shape
    # device layout [ω][J][I] = Fortran (I, J, ω): store the transpose of each matrix
    eps = torch.from_numpy(np.ascontiguousarray(P.transpose(0, 2, 1))).cuda()
    r = peps.eps_inverse(eps, N, nom, precision=precision, iters=iters, omega_batch=omega_batch)
    torch.cuda.synchronize()
    if r.status is not None:
        assert int(r.status.item()) == 0
    return eps.cpu().numpy().transpose(0, 2, 1)


def _rel(a, ref):
    return max(np.max(np.abs(a[w] - ref[w])) / np.max(np.abs(ref[w] + np.eye(ref.shape[1]))) for w in range(len(a)))


@pytest.mark.parametrize("N,nom,cond,batch", [(100, 3, 10.0, None), (300, 4, 300.0, 3), (256, 2, 1000.0, None)])
def test_refined_inverse_matches_fp64(N, nom, cond, batch):
    P = _problem(N, nom, cond)
    ref = _inverse_minus_one(P)
    e0 = _rel(_run(P, "mixed", iters=0, omega_batch=batch), ref)
    e1 = _rel(_run(P, "mixed", iters=1, omega_batch=batch), ref)
    e2 = _rel(_run(P, "mixed", iters=2, omega_batch=batch), ref)
    print(f"N={N} cond={cond}: FP32 {e0:.2e}, one step {e1:.2e}, two steps {e2:.2e}")
    assert e0 < 1e-2                        # FP32 inverse alone
    assert e1 < max(1e-9, 100 * e0 * e0)    # one step squares the error
    # floor of the split-precision residual: six 8-bit digits (2^-48 per value and
    # per dropped digit pair) summed over 2N products, times the condition number
    assert e2 < 1e-10, (e0, e1, e2)
    f64 = _rel(_run(P, "fp64"), ref)
    assert f64 < 1e-12


def test_mixed_inverse_q0_head_and_wings_match_fp64():
    N, nom = 160, 3
    P = _problem(N, nom, 50.0, seed=3)
    rng = np.random.default_rng(4)
    w1 = (rng.normal(size=(nom, N)) + 1j * rng.normal(size=(nom, N))) * 0.05
    head = rng.uniform(1.0, 3.0, size=nom) + 0.0j
    out = {}
    for prec in ("fp64", "mixed"):
        eps = torch.from_numpy(np.ascontiguousarray(P.transpose(0, 2, 1))).cuda()
        epsw1 = torch.from_numpy(w1.copy()).cuda()
        r = peps.eps_inverse(eps, N, nom, epsw1=epsw1, head=head, precision=prec)
        torch.cuda.synchronize()
        out[prec] = [t.cpu().numpy() for t in (r.eps, r.epsw1, r.epsw2, r.head)]
    for a, b in zip(out["mixed"], out["fp64"]):
        assert np.max(np.abs(a - b)) <= 1e-10 * max(1.0, np.max(np.abs(b)))
