"""ctypes bindings of libspi_engine.so (the C ABI of include/spi_engine.h).

There is no fallback: if the library is missing, loading fails with an error
that says how to build it.
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, c_double, c_float, c_int, c_int64, c_void_p

from ._build import ENGINE_SO, HOSTEMU_SO
from .robot import SpiRobot

SPI_OK = 0
ERRORS = {-1: "SPI_EINVAL", -2: "SPI_ENOMEM", -3: "SPI_ECUDA", -4: "SPI_ESTATE",
          -5: "SPI_ETIMEOUT", -6: "SPI_EBUDGET"}


class SpiError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


_engine = None
_hostemu = None

# name -> (restype, argtypes)
ENGINE_API = {
    "spi_abi_version": (c_int, []),
    "spi_last_error": (ctypes.c_char_p, []),
    "spi_create": (c_int, [POINTER(SpiRobot), POINTER(c_void_p)]),
    "spi_destroy": (c_int, [c_void_p]),
    "spi_set_stream": (c_int, [c_void_p, c_void_p]),
    "spi_load_windows": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_int, c_float]),
    "spi_set_theta": (c_int, [c_void_p, c_void_p, c_int]),
    "spi_set_cost": (c_int, [c_void_p, c_int, POINTER(c_float)]),
    "spi_run": (c_int, [c_void_p]),
    "spi_set_kernel_config": (c_int, [c_void_p, c_int]),
    "spi_set_kernel_layout": (c_int, [c_void_p, c_int]),
    "spi_run_trace": (c_int, [c_void_p, c_void_p]),
    "spi_read_costs": (c_int, [c_void_p, c_void_p, c_void_p]),
    "spi_sync": (c_int, [c_void_p, POINTER(c_int64)]),
    "spi_read_theta": (c_int, [c_void_p, c_void_p]),
    "spi_step_states": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_int]),
    "spi_sensitivity": (c_int, [c_void_p, c_void_p, c_int, POINTER(ctypes.c_int32), c_int, c_void_p, c_void_p]),
    "spi_fisher": (c_int, [c_void_p, c_int, c_int, c_int, c_void_p, c_double, c_void_p, c_void_p, c_void_p,
                           c_void_p]),
    "spi_fisher_ex": (c_int, [c_void_p, c_int, c_int, c_int, c_void_p, c_double, c_int, c_void_p, c_void_p,
                              c_void_p, c_void_p]),
    "spi_probe_fp32_peak": (c_int, [POINTER(c_double)]),
    "spi_adjoint": (c_int, [c_void_p, c_void_p, c_int, c_void_p, c_void_p]),
    "spi_search_create": (c_int, [c_void_p, c_void_p, POINTER(c_void_p)]),
    "spi_search_destroy": (c_int, [c_void_p]),
    "spi_search_sample": (c_int, [c_void_p, POINTER(c_void_p)]),
    "spi_search_refit": (c_int, [c_void_p, c_void_p]),
    "spi_search_read": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "spi_fd_fisher": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_int, POINTER(ctypes.c_int32), c_int,
                              c_float, c_int, c_int, c_void_p, c_void_p]),
    "spi_eval_windows_noalloc": (c_int, [POINTER(SpiRobot), c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_int,
                                         c_float, c_void_p, c_int, c_int, POINTER(c_float), c_void_p, c_void_p,
                                         c_void_p]),
}


def engine_lib():
    global _engine
    if _engine is None:
        if not ENGINE_SO.exists():
            raise SpiError(-4, f"{ENGINE_SO} is not built: run __graft_entry__.build() "
                               "(or spi_gb300._build.build()) first")
        lib = ctypes.CDLL(str(ENGINE_SO))
        for name, (res, args) in ENGINE_API.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        if lib.spi_abi_version() != 1:
            raise SpiError(-4, "libspi_engine.so ABI version mismatch")
        _engine = lib
    return _engine


def check(rc):
    if rc != SPI_OK:
        raise SpiError(rc, engine_lib().spi_last_error().decode(errors="replace"))
    return rc


def hostemu_lib():
    global _hostemu
    if _hostemu is None:
        if not HOSTEMU_SO.exists():
            raise SpiError(-4, f"{HOSTEMU_SO} is not built")
        lib = ctypes.CDLL(str(HOSTEMU_SO))
        lib.spi_hostemu_rollout.restype = c_int
        lib.spi_hostemu_rollout.argtypes = [POINTER(SpiRobot), c_void_p, c_void_p, c_void_p, c_int, c_int, c_void_p]
        lib.spi_hostemu_rollout_f32.restype = c_int
        lib.spi_hostemu_rollout_f32.argtypes = lib.spi_hostemu_rollout.argtypes
        lib.spi_hostemu_rollout_aba.restype = c_int
        lib.spi_hostemu_rollout_aba.argtypes = lib.spi_hostemu_rollout.argtypes
        lib.spi_hostemu_count_ops.restype = c_int
        lib.spi_hostemu_count_ops.argtypes = [POINTER(SpiRobot), c_void_p, c_void_p, c_void_p,
                                              POINTER(ctypes.c_longlong), POINTER(ctypes.c_longlong)]
        lib.spi_hostemu_count_ops_aba.restype = c_int
        lib.spi_hostemu_count_ops_aba.argtypes = lib.spi_hostemu_count_ops.argtypes
        lib.spi_hostemu_count_ops_dual.restype = c_int
        lib.spi_hostemu_count_ops_dual.argtypes = [POINTER(SpiRobot), c_void_p, c_void_p, c_void_p,
                                                   POINTER(ctypes.c_longlong)]
        lib.spi_hostemu_grad.restype = c_int
        lib.spi_hostemu_grad.argtypes = [POINTER(SpiRobot), c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int,
                                         c_int, c_int, c_void_p, c_void_p]
        lib.spi_hostemu_residual.restype = c_int
        lib.spi_hostemu_residual.argtypes = [POINTER(SpiRobot), c_void_p, c_void_p, c_void_p, c_void_p]
        _hostemu = lib
    return _hostemu
