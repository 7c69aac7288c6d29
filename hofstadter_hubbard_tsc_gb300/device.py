"""Python handles over the C ABI objects (context, operators, bases, waves)."""
import ctypes as C
import weakref

import numpy as np

from . import _lib
from .types import TotalBlock, SubBlock


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Device:
    """One library context = one GPU and one CUDA stream."""

    def __init__(self, device=0):
        self.lib = _lib.load()
        h = C.c_void_p()
        st = self.lib.hh_init(int(device), C.byref(h))
        if st != 0:
            raise _lib.HHError(st, "hh_init failed (no CUDA device?)")
        self.h = h
        self.device = device
        self.children = weakref.WeakSet()

    def adopt(self, obj):
        self.children.add(obj)
        return obj

    def check(self, st):
        _lib.check(st, self.h)

    def stream(self):
        s = C.c_void_p()
        self.check(self.lib.hh_ctx_stream(self.h, C.byref(s)))
        return s.value

    def sync(self):
        self.check(self.lib.hh_ctx_sync(self.h))

    def close(self):
        """Frees every live object of the context, then the context."""
        if self.h is not None:
            for obj in list(self.children):
                obj.free()
            self.lib.hh_finalize(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class DBlock:
    """Device-resident Total_Block."""

    def __init__(self, dev, handle, len, up_dif, down_dif, qn):
        self.dev, self.h = dev, handle
        self.len, self.up_dif, self.down_dif = len, up_dif, down_dif
        self.qn = qn  # (nsub, 5) int32
        dev.adopt(self)

    @classmethod
    def upload(cls, dev, blk: TotalBlock):
        qn = blk.qn_array()
        data = blk.data()
        h = C.c_void_p()
        dev.check(dev.lib.hh_block_create(dev.h, blk.len, blk.up_dif, blk.down_dif, blk.num, _ip(qn),
                                          _dp(data), C.byref(h)))
        return cls(dev, h, blk.len, blk.up_dif, blk.down_dif, qn[:blk.num].copy())

    @classmethod
    def from_handle(cls, dev, h):
        """Wraps a block the library created (takes ownership)."""
        ln, up, dn, ns = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        dev.check(dev.lib.hh_block_info(h, C.byref(ln), C.byref(up), C.byref(dn), C.byref(ns), None))
        qn = np.zeros((max(1, ns.value), 5), dtype=np.int32)
        if ns.value:
            dev.check(dev.lib.hh_block_qn(h, _ip(qn)))
        return cls(dev, h, ln.value, up.value, dn.value, qn[:ns.value].copy())

    @classmethod
    def zeros_like(cls, other):
        dev = other.dev
        h = C.c_void_p()
        qn = np.ascontiguousarray(other.qn if len(other.qn) else np.zeros((1, 5), np.int32))
        dev.check(dev.lib.hh_block_zeros(dev.h, other.len, other.up_dif, other.down_dif, len(other.qn),
                                         _ip(qn), C.byref(h)))
        return cls(dev, h, other.len, other.up_dif, other.down_dif, other.qn.copy())

    def add(self, coef, src):
        """self += coef * src (block_add_block_two, code/space_info.f90:176-214)."""
        c = np.array([complex(coef).real, complex(coef).imag], dtype=np.float64)
        self.dev.check(self.dev.lib.hh_block_add(self.h, _dp(c), src.h))

    def download(self):
        n = C.c_longlong()
        self.dev.check(self.dev.lib.hh_block_info(self.h, None, None, None, None, C.byref(n)))
        buf = np.zeros(max(1, 2 * n.value), dtype=np.float64)
        self.dev.check(self.dev.lib.hh_block_download(self.h, _dp(buf)))
        z = buf.view(np.complex128)
        subs, o = [], 0
        for (up, down, dd, r, c) in self.qn:
            subs.append(SubBlock(up, down, dd, z[o:o + r * c].reshape((r, c), order="F").copy()))
            o += r * c
        return TotalBlock(self.len, self.up_dif, self.down_dif, subs)

    def free(self):
        if self.h is not None and self.dev.h is not None:
            self.dev.lib.hh_block_free(self.h)
        self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class DBasis:
    def __init__(self, dev, basis):
        self.dev = dev
        sec, sub = basis.arrays()
        h = C.c_void_p()
        dev.check(dev.lib.hh_basis_create(dev.h, basis.len, basis.num, _ip(sec), _ip(sub), C.byref(h)))
        self.h = h
        self.host = basis
        dev.adopt(self)

    def free(self):
        if self.h is not None and self.dev.h is not None:
            self.dev.lib.hh_basis_free(self.h)
        self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class DWave:
    """Device-resident Wavefunction (nbatch vectors sharing one layout)."""

    def __init__(self, dev, layout, sys_len, env_len, nbatch=1):
        self.dev = dev
        self.layout = np.ascontiguousarray(layout, dtype=np.int32)
        h = C.c_void_p()
        dev.check(dev.lib.hh_wave_create(dev.h, sys_len, env_len, len(self.layout), _ip(self.layout),
                                         int(nbatch), C.byref(h)))
        self.h = h
        dev.adopt(self)
        self.nbatch = nbatch
        self.sys_len, self.env_len = sys_len, env_len
        self.nelem = int(sum(int(r[4]) * int(r[5]) for r in self.layout))

    def upload(self, z):
        z = np.ascontiguousarray(np.asarray(z, dtype=np.complex128).ravel())
        assert z.size == self.nelem * self.nbatch
        self.dev.check(self.dev.lib.hh_wave_upload(self.h, _dp(z.view(np.float64))))

    def download(self):
        z = np.zeros(max(1, self.nelem * self.nbatch), dtype=np.complex128)
        self.dev.check(self.dev.lib.hh_wave_download(self.h, _dp(z.view(np.float64))))
        return z[:self.nelem * self.nbatch]

    def norm(self):
        r = C.c_double()
        self.dev.check(self.dev.lib.hh_wave_norm(self.h, C.byref(r)))
        return r.value

    def dot(self, other):
        r = C.c_double()
        self.dev.check(self.dev.lib.hh_wave_dot(self.h, other.h, C.byref(r)))
        return r.value

    def free(self):
        if self.h is not None and self.dev.h is not None:
            self.dev.lib.hh_wave_free(self.h)
        self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

