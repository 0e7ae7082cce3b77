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
