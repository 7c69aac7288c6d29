"""Ground-state Lanczos ``lanczos_memo_new`` (code/lanczos.f90:4-177), levels=1.

Three-term recurrence with alpha = Re<v,Hv>, beta = ||r|| before
normalisation, breakdown when beta <= lanzero (code/lanczos.f90:77-80), full
Gram-Schmidt of the new vector against all previous Krylov vectors with the
real inner product (code/lanczos.f90:85), the lowest Ritz value of the
tridiagonal matrix at every step (DSTEV 'N', code/lanczos.f90:96-99) and
convergence when it moves by <= lanzero or after loop_in=100 vectors
(code/lanczos.f90:102).  The outer restart at code/lanczos.f90:115-136 is
unreachable (iter_out equals loop_out on the first pass), so only the exit at
label 411 is restated: psi = sum_i z_i v_i, normalised.
"""
import numpy as np
from scipy.linalg import eigh_tridiagonal

from .blocks import wave_product, wave_norm, wave_normalize, gram_schmidt_process

LOOP_IN = 100


def tridiag_lowest(alpha, beta, vectors=False):
    """Lowest eigenpair of the symmetric tridiagonal (alpha, beta[:-1])."""
    n = len(alpha)
    if n == 1:
        return (alpha[0], np.ones(1)) if vectors else alpha[0]
    e = np.asarray(beta[:n - 1], dtype=np.float64)
    if vectors:
        w, z = eigh_tridiagonal(np.asarray(alpha, dtype=np.float64), e)
        return w[0], z[:, 0]
    w = eigh_tridiagonal(np.asarray(alpha, dtype=np.float64), e, eigvals_only=True)
    return w[0]


def lanczos_memo_new(apply_h, eigvec, lanzero, loop_in=LOOP_IN, log=None):
    """Returns (E0, iterations) and overwrites eigvec with the ground state.

    ``apply_h(v, out)`` evaluates model_wave(v) into ``out`` (both Wave).
    """
    v = [eigvec.copy()]
    wave_normalize(v[0])
    last = 1
    alpha = []
    beta = []
    w = v[0].zeros_like()
    apply_h(v[0], w)
    alpha.append(wave_product(v[0], w))
    ritzmin = alpha[0]
    while last < loop_in:
        for i, ws in enumerate(w.subs):
            if last < 2:
                ws.vec = ws.vec - alpha[last - 1] * v[last - 1].subs[i].vec
            else:
                ws.vec = (ws.vec - alpha[last - 1] * v[last - 1].subs[i].vec
                          - beta[last - 2] * v[last - 2].subs[i].vec)
        b = wave_norm(w)
        beta.append(b)
        if abs(b) <= lanzero:
            break
        wave_normalize(w)
        gram_schmidt_process(v[:last], w)
        v.append(w)
        last += 1
        w = v[0].zeros_like()
        apply_h(v[last - 1], w)
        alpha.append(wave_product(v[last - 1], w))
        d0 = tridiag_lowest(alpha[:last], (beta + [0.0])[:last])
        if log is not None:
            log.append(d0)
        if abs(d0 - ritzmin) <= lanzero or last == loop_in:
            ritzmin = d0
            break
        ritzmin = d0
    bb = (beta + [0.0] * (last + 1))[:last]
    e0, z = tridiag_lowest(alpha[:last], bb, vectors=True)
    for ws in eigvec.subs:
        ws.vec = np.zeros_like(ws.vec)
    for i in range(last):
        for x, ws in enumerate(eigvec.subs):
            ws.vec = ws.vec + z[i] * v[i].subs[x].vec
    wave_normalize(eigvec)
    return float(e0), last
