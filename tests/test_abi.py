"""The C-ABI library loads and exports every entry point declared in include/*.h (no GPU needed)."""
import ctypes
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names.update(re.findall(r"^\s*(?:const\s+)?[\w\*\s]+?\b(spi_\w+)\s*\(", text, flags=re.M))
    return sorted(names)


def test_library_exports_every_declared_symbol(built):
    from spi_gb300._build import ENGINE_SO
    lib = ctypes.CDLL(str(ENGINE_SO))
    names = declared_symbols()
    assert "spi_run" in names and "spi_create" in names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_abi_version_and_struct_size(built):
    from spi_gb300 import _lib
    from spi_gb300.robot import SpiRobot
    lib = _lib.engine_lib()
    assert lib.spi_abi_version() == 1
    # 12*3 + 12 + 12*3 + 12*6 + 1+3+6 + 1+3+6 + 3+1 + 24 + 4 + 24 + 4 + 36 + 3+3+1 + 2 floats, 4 ints
    assert ctypes.sizeof(SpiRobot) == 4 * (36 + 12 + 36 + 72 + 10 + 10 + 4 + 24 + 5 + 24 + 4 + 36 + 7 + 2 + 4)


def test_errors_are_reported_without_gpu(built):
    from spi_gb300 import _lib
    lib = _lib.engine_lib()
    rc = lib.spi_run(None)
    assert rc == -1
    assert b"null engine" in lib.spi_last_error()
    rc = lib.spi_create(None, None)
    assert rc == -1


def test_kernel_variant_and_fisher_entry_points_validate_arguments(built):
    """Null handles and out-of-range arguments come back as SPI_EINVAL before any CUDA call."""
    import ctypes
    from spi_gb300 import _lib
    from spi_gb300.server import _bind
    lib = _lib.engine_lib()
    assert lib.spi_set_kernel_layout(None, 1) == -1
    assert lib.spi_set_kernel_config(None, 3) == -1
    assert lib.spi_fisher_ex(None, 1, 1, 13, None, ctypes.c_double(0.0), 1, None, None, None, None) == -1
    assert b"spi_fisher" in lib.spi_last_error()
    assert lib.spi_fisher_ex(None, 1, 1, 14, None, ctypes.c_double(0.0), 0, None, None, None, None) == -1
    srv = _bind(ctypes.CDLL(lib._name))
    assert srv.spi_server_set_kernel_layout(None, 1) == -1
    assert srv.spi_server_set_kernel_config(None, 3) == -1


def test_model_builder_rejects_unsupported_joint_origins(built):
    """The kernel's transforms take hip joint origins in the base's x-y plane, thigh origins
    on the hip frame's y axis, calf origins and the foot on the thigh's and the calf's z axes;
    the model builder (shared by the engine and the host emulation) refuses any other robot
    with SPI_EINVAL."""
    import numpy as np
    from spi_gb300 import _lib
    from spi_gb300.data import standing_state
    from spi_gb300.robot import SimConfig, THETA_NOMINAL, to_struct
    lib = _lib.hostemu_lib()
    x = np.ascontiguousarray(standing_state(1), dtype=np.float64)
    th = np.ascontiguousarray(THETA_NOMINAL[None], dtype=np.float64)
    a = np.zeros((1, 1, 12))
    out = np.zeros((1, 1, 37))

    def run(r):
        return lib.spi_hostemu_rollout(ctypes.byref(r), x.ctypes.data, a.ctypes.data, th.ctypes.data, 1, 1,
                                       out.ctypes.data)

    assert run(to_struct(SimConfig())) == 0
    for body, comp in ((0, 2), (1, 0), (7, 2), (2, 1), (11, 0)):   # body 3 leg + k: hip z, thigh x / z, calf y / x
        r = to_struct(SimConfig())
        r.body_origin[body][comp] = 0.01
        assert run(r) == -1, (body, comp)
    for comp in (0, 1):                                              # the foot off the calf's z axis
        r = to_struct(SimConfig())
        r.foot[comp] = 0.01
        assert run(r) == -1, comp


def test_gradient_fd_fisher_and_search_entry_points_validate_arguments(built):
    """spi_adjoint, spi_fd_fisher and spi_search_* refuse null handles and out-of-range sizes with
    SPI_EINVAL before any CUDA call (no GPU needed)."""
    import ctypes
    from spi_gb300 import _lib
    from spi_gb300.cem import SpiCemConfig
    lib = _lib.engine_lib()
    assert lib.spi_adjoint(None, None, 4, None, None) == -1
    assert b"spi_adjoint" in lib.spi_last_error()
    ids = (ctypes.c_int32 * 2)(0, 1)
    assert lib.spi_fd_fisher(None, None, None, None, 4, 10, ids, 2, 0.1, 5, 1, None, None) == -1
    assert b"spi_fd_fisher" in lib.spi_last_error()
    out = ctypes.c_void_p()
    cfg = SpiCemConfig()
    cfg.n_samples, cfg.dim = 1, 2          # fewer than two samples
    assert lib.spi_search_create(ctypes.byref(cfg), None, ctypes.byref(out)) == -1
    assert b"n_samples" in lib.spi_last_error()
    cfg.n_samples, cfg.dim = 64, 14        # more than 13 dimensions
    assert lib.spi_search_create(ctypes.byref(cfg), None, ctypes.byref(out)) == -1
    cfg.dim = 2
    cfg.param_ids[0], cfg.param_ids[1] = 3, 3
    cfg.lo[0], cfg.hi[0], cfg.lo[1], cfg.hi[1] = 0.0, 1.0, 0.0, 1.0
    cfg.elite_frac, cfg.alpha = 0.1, 1.0
    assert lib.spi_search_create(ctypes.byref(cfg), None, ctypes.byref(out)) == -1   # repeated slot
    assert b"repeated" in lib.spi_last_error()
    assert lib.spi_search_sample(None, None) == -1
    assert lib.spi_search_refit(None, None) == -1
