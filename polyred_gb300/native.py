"""Loader for libpolyred_cuda.so (the CUDA render path).

The library is built in-tree (polyred_gb300/lib/) by polyred_gb300.build;
POLYRED_CUDA_LIB names another build of it to load instead (as the Go
binding's variable of that name does). There is no fallback: if the library
cannot be loaded, every render call raises NativeUnavailable.
"""
import ctypes as C
import os

from . import _abi

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lib", "libpolyred_cuda.so")

_lib = None


class NativeUnavailable(RuntimeError):
    """libpolyred_cuda.so is missing or failed to load."""


class RenderError(RuntimeError):
    """A pr_* entry point returned an error status."""

    def __init__(self, status, detail):
        super().__init__(f"{detail} (status {status})")
        self.status = status


def load(build_if_missing=False):
    """Return the bound CDLL, building it first when asked."""
    global _lib
    if _lib is not None:
        return _lib
    path = os.environ.get("POLYRED_CUDA_LIB")
    if path:
        return _open(path)
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise NativeUnavailable(f"{LIB_PATH} not built; run polyred_gb300.build.build()")
        from . import build
        build.build()
    return _open(LIB_PATH)


def _open(path):
    global _lib
    try:
        lib = C.CDLL(path)
    except OSError as e:
        raise NativeUnavailable(f"cannot load {path}: {e}") from e
    _abi.bind(lib)
    if lib.pr_abi_version() != _abi.ABI_VERSION:
        raise NativeUnavailable("ABI version mismatch")
    _lib = lib
    return lib


def check(status):
    if status != _abi.PR_OK:
        lib = load()
        detail = lib.pr_last_error().decode(errors="replace") or lib.pr_error_string(status).decode()
        raise RenderError(status, detail)
    return status
