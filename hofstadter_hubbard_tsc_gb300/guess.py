"""Learned initial-guess corrector (no counterpart in the reference).

The reference starts every Lanczos run of a sweep from the transformed ground
state of the previous step (wave_trans_LR/RL, code/warm_up.f90:1855-2170).
``LearnedGuess`` rescales that guess sector by sector before the Lanczos run:
a small MLP (features -> 64 -> 64 -> 1, tanh, FP32; trained on the GPU by the
library's own kernels) predicts how much weight each symmetry sector of the
superblock will carry in the converged state, from

  0  log10 weight of the sector in the transformed guess
  1  log10 weight the sector had when this superblock position last converged
     (the guess weight when there is none)
  2  1 when that previous weight exists, else 0
  3  sys electron number / N_e
  4  sys 2S / 8,  5  env 2S / 8
  6  log(sys dim + 1) / 8,  7  log(env dim + 1) / 8
  8  sys length / number of sites

(log10 weights are floored at 1e-14 and divided by 14).  The target is the
change of the log10 weight from the guess to the converged state; the scale
applied to a sector's amplitudes is 10^(14 delta / 2), clipped to [0.5, 2],
and only sectors carrying at least 1e-6 of the guess's weight are rescaled
(amplifying the rest injects noise and costs iterations).  Training pairs
(guess features, converged weights) come from every step of the earlier
sweeps that started from a transformed guess.

Training weights each sample by the sector's weight, max(w_converged,
w_guess), so that the loss follows the Hellinger distance between sector
weight distributions, which bounds what a rescaling does to the guess's
infidelity.  The plain transformed guess stays the fallback: every fifth
recorded step is held out of training, and the network is applied only while
the corrected weights of the held-out steps are closer to the converged ones
than the plain guess's, in summed Hellinger distance
sum_k (sqrt(w_converged) - sqrt(w))^2, by a factor 0.8.  With ``rq_check``
the corrected guess must also have a lower Rayleigh quotient than the plain
one (two extra matvecs per step).

Measured ceiling (2x8 m=64 and 2x16 m=256 Hubbard ladders, phi = 1/4): a
Lanczos run started from the guess rescaled to the exact converged sector
weights needs 0.7-1.3 % fewer iterations, and one started from the best
per-sector combination a_k g_k + b_k r_k of the guess g and its residual r
about 3 % fewer: the guess error lies inside the sectors.
"""
import ctypes as C
import time

import numpy as np

from . import _lib

NFEAT = 9
_FLOOR = 1e-14


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class SectorMLP:
    """The corrector's network on the device (hh_mlp_*)."""

    def __init__(self, dev, nfeat=NFEAT, seed=20261203):
        self.dev, self.nfeat = dev, nfeat
        h = C.c_void_p()
        dev.check(dev.lib.hh_mlp_create(dev.h, nfeat, C.c_ulonglong(seed), C.byref(h)))
        self.h = h
        n = C.c_int()
        dev.check(dev.lib.hh_mlp_nparams(h, C.byref(n)))
        self.nparams = n.value

    def get_params(self):
        p = np.zeros(self.nparams, dtype=np.float32)
        self.dev.check(self.dev.lib.hh_mlp_get_params(self.h, _fp(p)))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.nparams
        self.dev.check(self.dev.lib.hh_mlp_set_params(self.h, _fp(p)))

    def forward(self, X):
        X = np.ascontiguousarray(X, dtype=np.float32)
        y = np.zeros(len(X), dtype=np.float32)
        if len(X):
            self.dev.check(self.dev.lib.hh_mlp_forward(self.h, _fp(X), len(X), _fp(y)))
        return y

    def _xtw(self, X, T, W):
        X = np.ascontiguousarray(X, dtype=np.float32)
        T = np.ascontiguousarray(T, dtype=np.float32)
        W = None if W is None else np.ascontiguousarray(W, dtype=np.float32)
        assert X.shape == (len(T), self.nfeat)
        return X, T, W

    def loss_grad(self, X, T, W=None):
        X, T, W = self._xtw(X, T, W)
        loss = np.zeros(1, dtype=np.float32)
        g = np.zeros(self.nparams, dtype=np.float32)
        self.dev.check(self.dev.lib.hh_mlp_loss_grad(self.h, _fp(X), _fp(T), None if W is None else _fp(W),
                                                     len(T), _fp(loss), _fp(g)))
        return float(loss[0]), g

    def train(self, X, T, W=None, epochs=400, lr=3e-3):
        X, T, W = self._xtw(X, T, W)
        loss = np.zeros(1, dtype=np.float32)
        self.dev.check(self.dev.lib.hh_mlp_train(self.h, _fp(X), _fp(T), None if W is None else _fp(W), len(T),
                                                 int(epochs), C.c_float(lr), _fp(loss)))
        return float(loss[0])

    def free(self):
        if getattr(self, "h", None) is not None and self.dev.h is not None:
            self.dev.lib.hh_mlp_free(self.h)
        self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def sector_norms(dev, w):
    """Squared norm of every sector of a device wave."""
    n = len(w.layout)
    out = np.zeros(max(1, n))
    dev.check(dev.lib.hh_wave_sector_norms(w.h, out.ctypes.data_as(C.POINTER(C.c_double))))
    return out[:n]


def scale_sectors(dev, w, scale):
    s = np.ascontiguousarray(scale, dtype=np.float64)
    assert s.size == len(w.layout)
    dev.check(dev.lib.hh_wave_scale_sectors(w.h, s.ctypes.data_as(C.POINTER(C.c_double))))


def _lw(w):
    return np.log10(np.maximum(w, 0.0) + _FLOOR) / 14.0


class LearnedGuess:
    """guess_hook of ``GPUDMRG``: records training pairs, trains between
    sweeps (``end_sweep``) and corrects transformed guesses once trained.

    ``apply=False`` records and trains but never changes a guess (the plain
    method with the same bookkeeping)."""

    def __init__(self, dev, n_sites, n_elec, seed=20261203, apply=True, min_samples=64, epochs=400, lr=3e-3,
                 rq_check=False, mlp=None):
        """mlp: the network (SectorMLP on dev when None; anything with its
        forward / train / free methods otherwise)."""
        self.dev, self.n_sites, self.n_elec = dev, n_sites, n_elec
        self.mlp = SectorMLP(dev, NFEAT, seed) if mlp is None else mlp
        self.apply = apply
        self.min_samples, self.epochs, self.lr = min_samples, epochs, lr
        self.X, self.T, self.W = [], [], []
        self.WG, self.WC = [], []     # guess and converged sector weights per recorded step
        self.prev = {}            # (sys_len, env_len) -> {sector qn: converged weight}
        self.rq_check = rq_check
        self.trained = False          # network trained at least once
        self.enabled = False          # held-out error below the gate
        self.train_s = 0.0
        self.last_loss = None
        self.val = None               # held-out Hellinger distance (corrected, plain)
        self.val_history = []         # self.val of every training
        self.log = []             # (sys_len, env_len, used_corrected, rq_plain, rq_corrected)
        self._pending = None

    # ------------------------------------------------------------ features
    def features(self, key, subs, wg):
        sys_len, env_len = key
        prev = self.prev.get(key)
        X = np.zeros((len(subs), NFEAT))
        X[:, 0] = _lw(wg)
        for k, s in enumerate(subs):
            qn = (s.sys_num_up, s.sys_num_down, s.env_num_up, s.env_num_down)
            if prev is not None and qn in prev:
                X[k, 1] = _lw(prev[qn])
                X[k, 2] = 1.0
            else:
                X[k, 1] = X[k, 0]
            X[k, 3] = s.sys_num_up / max(1, self.n_elec)
            X[k, 4] = s.sys_num_down / 8.0
            X[k, 5] = s.env_num_down / 8.0
            X[k, 6] = np.log(s.sys_dim + 1.0) / 8.0
            X[k, 7] = np.log(s.env_dim + 1.0) / 8.0
            X[k, 8] = sys_len / self.n_sites
        return X

    # ---------------------------------------------------------------- hook
    def __call__(self, dmrg, sb, psi, when):
        key = (sb.sys.len, sb.env.len)
        subs = sb.sup.subs
        if when == "before":
            kind = getattr(dmrg, "guess_kind", "transformed")
            wg = sector_norms(self.dev, psi)
            wg = wg / max(wg.sum(), 1e-300)
            X = self.features(key, subs, wg)
            self._pending = (key, X, wg, kind == "transformed")
            if kind == "transformed" and self.enabled and self.apply:
                self._correct(sb, psi, X, wg)
            return
        # after: converged weights -> training pair, previous-weight table
        wc = sector_norms(self.dev, psi)
        wc = wc / max(wc.sum(), 1e-300)
        pk, X, wg, transformed = self._pending
        self._pending = None
        if pk == key and transformed:
            self.X.append(X)
            self.T.append(_lw(wc) - X[:, 0])
            self.W.append(np.maximum(wc, wg) + 1e-8)
            self.WG.append(wg)
            self.WC.append(wc)
        self.prev[key] = {(s.sys_num_up, s.sys_num_down, s.env_num_up, s.env_num_down): float(wc[k])
                          for k, s in enumerate(subs)}

    def _correct(self, sb, psi, X, wg):
        delta = self.mlp.forward(X).astype(np.float64)
        if not np.all(np.isfinite(delta)):
            self.log.append((sb.sys.len, sb.env.len, False, None, None))
            return
        scale = self.scales(delta, wg)
        dev = self.dev
        if not self.rq_check:
            scale_sectors(dev, psi, scale)
            dev.check(dev.lib.hh_wave_normalize(psi.h))
            self.log.append((sb.sys.len, sb.env.len, True, None, None))
            return
        # Rayleigh quotients of the plain and the corrected guess
        sb.matvec(psi, sb.w_out)
        rq_plain = psi.dot(sb.w_out) / psi.dot(psi)
        dev.check(dev.lib.hh_wave_copy(sb.w_in.h, psi.h))
        scale_sectors(dev, sb.w_in, scale)
        dev.check(dev.lib.hh_wave_normalize(sb.w_in.h))
        sb.matvec(sb.w_in, sb.w_out)
        rq_corr = sb.w_in.dot(sb.w_out)
        use = bool(np.isfinite(rq_corr) and rq_corr < rq_plain)
        if use:
            dev.check(dev.lib.hh_wave_copy(psi.h, sb.w_in.h))
        self.log.append((sb.sys.len, sb.env.len, use, rq_plain, rq_corr))

    # ------------------------------------------------------------ training
    def data(self, held_out=None):
        """Recorded pairs; held_out True/False selects every fifth step or the rest."""
        steps = [k for k in range(len(self.X)) if held_out is None or ((k % 5 == 4) == held_out)]
        if not steps:
            return np.zeros((0, NFEAT)), np.zeros(0), np.zeros(0)
        return (np.concatenate([self.X[k] for k in steps]), np.concatenate([self.T[k] for k in steps]),
                np.concatenate([self.W[k] for k in steps]))

    @staticmethod
    def scales(delta, wg):
        """Amplitude scale per sector from the predicted log10-weight change."""
        return np.where(wg >= 1e-6, np.clip(10.0 ** (14.0 * np.asarray(delta, dtype=np.float64) / 2.0), 0.5, 2.0),
                        1.0)

    def train(self):
        X, T, W = self.data(held_out=False)
        held = [k for k in range(len(self.X)) if k % 5 == 4]
        if len(T) < self.min_samples or not held:
            return None
        t0 = time.perf_counter()
        self.last_loss = self.mlp.train(X, T, W, epochs=self.epochs, lr=self.lr)
        h_net = h_plain = 0.0
        for k in held:
            wg, wc = self.WG[k], self.WC[k]
            w = wg * self.scales(self.mlp.forward(self.X[k]), wg) ** 2
            w /= max(w.sum(), 1e-300)
            h_net += float(np.sum((np.sqrt(wc) - np.sqrt(w)) ** 2))
            h_plain += float(np.sum((np.sqrt(wc) - np.sqrt(wg)) ** 2))
        self.train_s += time.perf_counter() - t0
        self.val = (h_net, h_plain)
        self.val_history.append(self.val)
        self.trained = True
        self.enabled = h_net < 0.8 * h_plain
        return self.last_loss

    def end_sweep(self, dmrg):
        self.train()

    def free(self):
        self.mlp.free()
