"""Reduced density matrix and per-sector truncation (code/get_den.f90).

Eigenvectors returned by LAPACK are defined up to a phase (and up to a unitary
inside degenerate subspaces), so results that compare across implementations
are the kept eigenvalues, the discarded weight, the entropy and gauge-invariant
products such as T T^H.  ``canonical_phase`` fixes one phase convention (the
largest-modulus component of every eigenvector real and positive) so that the
oracle and the GPU path can be compared column by column where the spectrum is
non-degenerate.
"""
import numpy as np

from .blocks import Block, Sub


def get_density_matrix_sys(wave):
    """rho_s = psi psi^H per sector (code/get_den.f90:4-49)."""
    den = Block(wave.sys_len, 0, 0)
    for w in wave.subs:
        den.subs.append(Sub(w.sys_num_up, w.sys_num_down, 0, w.sys_dim, w.sys_dim,
                            w.vec @ np.conj(w.vec).T))
    return den


def get_density_matrix_env(wave):
    """rho_e = psi^H psi per sector (code/get_den.f90:55-99)."""
    den = Block(wave.env_len, 0, 0)
    for w in wave.subs:
        den.subs.append(Sub(w.env_num_up, w.env_num_down, 0, w.env_dim, w.env_dim,
                            np.conj(w.vec).T @ w.vec))
    return den


def quicksort_double(arr, idx, lower, upper):
    """Descending quicksort with index tracking (code/update.f90:322-368).

    Restated exactly (middle pivot, Hoare partition) so that the order of equal
    eigenvalues, and therefore which of several degenerate states is kept at
    the cut, matches the reference.  ``lower``/``upper`` are 0-based inclusive.
    """
    stack = [(lower, upper)]
    while stack:
        lo, hi = stack.pop()
        i, j = lo, hi
        pivot = arr[(lo + hi + 2) // 2 - 1]  # Fortran int((lower+upper)/2) on 1-based indices
        while i <= j:
            while arr[i] > pivot:
                i += 1
            while arr[j] < pivot:
                j -= 1
            if i <= j:
                arr[i], arr[j] = arr[j], arr[i]
                idx[i], idx[j] = idx[j], idx[i]
                i += 1
                j -= 1
        # the reference recurses on (lower, j) first, then (i, upper)
        if i < hi:
            stack.append((i, hi))
        if lo < j:
            stack.append((lo, j))


def canonical_phase(vecs):
    """Rotate each column so its largest-modulus entry is real and positive."""
    if vecs.size == 0:
        return vecs
    k = np.argmax(np.abs(vecs), axis=0)
    ph = vecs[k, np.arange(vecs.shape[1])]
    ph = ph / np.abs(ph)
    return vecs / ph[None, :]


def get_truncation_operator(den, kept_min, kept_max, trun_err, phase_fix=True):
    """Get_truncation_operator (code/get_den.f90:184-428).

    Returns (trun Block, num_state, discarded weight tmp_err, entropy, spectrum).
    Per-sector ZHEEV (ascending), global descending sort, renormalisation to
    trace 1, selection from kept_min until the discarded weight is <= trun_err
    or kept_max is reached, entropy over eigenvalues >= 1e-15, and per sector
    the top eigenvectors in ascending order (columns row-col+1..row).
    """
    evals, evecs = [], []
    for s in den.subs:
        w, v = np.linalg.eigh(s.mat)
        if phase_fix:
            v = canonical_phase(v)
        evals.append(w)
        evecs.append(v)
    allv = np.concatenate(evals) if evals else np.zeros(0)
    gid = []
    off = 0
    for w in evals:
        gid.extend(range(off + 1, off + len(w) + 1))
        off += len(w)
    arr = list(allv.astype(float))
    idx = list(gid)
    n = len(arr)
    if n:
        quicksort_double(arr, idx, 0, n - 1)
    tot = sum(arr)
    arr = [a / tot for a in arr]
    if n <= kept_min:
        num_state = n
        tmp_err = 0.0
    else:
        tmp_err = sum(arr[kept_min:])
        num_state = kept_min
        while tmp_err > trun_err:
            num_state += 1
            tmp_err -= arr[num_state - 1]
            if tmp_err <= trun_err or num_state >= kept_max:
                break
    ent = 0.0
    for a in arr:
        if a >= 1.0e-15:
            ent -= a * np.log(a)
    kept_ids = set(idx[:num_state])
    # count kept states per sector (global ids are contiguous per sector)
    trun = Block(den.len, den.up_dif, den.down_dif)
    off = 0
    for s, w, v in zip(den.subs, evals, evecs):
        ncol = sum(1 for g in range(off + 1, off + len(w) + 1) if g in kept_ids)
        off += len(w)
        if ncol > 0:
            row = s.sdim
            trun.subs.append(Sub(s.num_up, s.num_down, 0, row, ncol,
                                 v[:, row - ncol:row].astype(np.complex128)))
    return trun, num_state, tmp_err, ent, np.array(arr)


def identity_truncation(basis):
    """block_transfer_basis + unit matrices (code/warm_up.f90:1432-1439)."""
    trun = Block(basis.len, 0, 0)
    for sec in basis.sectors:
        trun.subs.append(Sub(sec.new_num_up, sec.new_num_down, 0, sec.dim, sec.dim,
                             np.eye(sec.dim, dtype=np.complex128)))
    return trun
