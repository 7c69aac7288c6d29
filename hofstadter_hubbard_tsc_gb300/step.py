"""Density matrix, truncation, renormalisation and wavefunction transformation
behind the reference's subroutine names (code/get_den.f90, code/update.f90:
1387-1605, code/warm_up.f90:1855-2170); all arithmetic runs in libhh_dmrg.so."""
import ctypes as C

import numpy as np

from . import _lib
from .device import DBlock

SYS, ENV = 0, 1


def density_truncate(dev, wave, side, kept_min, kept_max, trun_err):
    """Get_density_matrix_{sys,env}_new + Get_truncation_operator for levels = 1.

    Returns (trun DBlock, num_state, discarded weight, entropy, sorted spectrum)."""
    h = C.c_void_p()
    ns, err, ent = C.c_int(), C.c_double(), C.c_double()
    dim = int(sum(int(r[4] if side == SYS else r[5]) for r in wave.layout))
    spec = np.zeros(max(1, dim))
    dev.check(dev.lib.hh_density_truncate(dev.h, wave.h, int(side), int(kept_min), int(kept_max), float(trun_err),
                                          C.byref(h), C.byref(ns), C.byref(err), C.byref(ent),
                                          spec.ctypes.data_as(C.POINTER(C.c_double))))
    return DBlock.from_handle(dev, h), ns.value, err.value, ent.value, spec[:dim]


def update_trun(dev, op, trun, dia, precision=_lib.HH_PREC_FP64):
    """update_trun_dia (dia=True) / update_trun_ndia: T^H O T.

    precision: HH_PREC_FP64 (the reference's arithmetic) or HH_PREC_FP32X2
    (double-float, the block operators of a split-precision sweep); set on
    the context for every call."""
    dev.check(dev.lib.hh_ctx_set_renormalize_precision(dev.h, int(precision)))
    h = C.c_void_p()
    dev.check(dev.lib.hh_renormalize(dev.h, op.h, trun.h, 1 if dia else 0, C.byref(h)))
    return DBlock.from_handle(dev, h)


def wave_trans(dev, direction, sys_bs, env_bs, sys_trun, env_trun, old_wave, new_wave, precision=_lib.HH_PREC_FP64):
    """wave_trans_LR (direction 'LR') / wave_trans_RL ('RL') into new_wave (normalised).

    precision: HH_PREC_FP64 (the reference's arithmetic) or HH_PREC_FP32 (the
    Lanczos start vector of a split-precision sweep); it is set on the context
    for every call, so no earlier call's choice carries over."""
    d = 0 if direction == "LR" else 1
    dev.check(dev.lib.hh_ctx_set_transform_precision(dev.h, int(precision)))
    dev.check(dev.lib.hh_wave_transform(dev.h, d, sys_bs.h, env_bs.h, sys_trun.h, env_trun.h, old_wave.h,
                                        new_wave.h))
    return new_wave
