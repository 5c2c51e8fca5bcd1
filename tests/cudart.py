"""Minimal ctypes access to the CUDA runtime for tests that hand device
buffers to the C ABI (device memory owned by the caller)."""
from __future__ import annotations

import ctypes as C
import glob
import os

_rt = None


def rt() -> C.CDLL:
    global _rt
    if _rt is None:
        home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
        cands = [os.path.join(home, "lib64", "libcudart.so")]
        cands += sorted(glob.glob(os.path.join(home, "targets", "*", "lib", "libcudart.so*")))
        cands += ["libcudart.so", "libcudart.so.13", "libcudart.so.12"]
        last = None
        for c in cands:
            try:
                _rt = C.CDLL(c)
                break
            except OSError as e:
                last = e
        if _rt is None:
            raise OSError(f"libcudart not found: {last}")
        _rt.cudaMalloc.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
        _rt.cudaFree.argtypes = [C.c_void_p]
        _rt.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
        _rt.cudaMemset.argtypes = [C.c_void_p, C.c_int, C.c_size_t]
        _rt.cudaSetDevice.argtypes = [C.c_int]
        _rt.cudaMemGetInfo.argtypes = [C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]
    return _rt


def _ck(code: int, what: str) -> None:
    if code != 0:
        raise RuntimeError(f"{what} failed with CUDA error {code}")


class DeviceBuffer:
    def __init__(self, nbytes: int):
        self.nbytes = nbytes
        self.ptr = C.c_void_p()
        _ck(rt().cudaMalloc(C.byref(self.ptr), nbytes), "cudaMalloc")

    def upload(self, arr) -> None:
        assert arr.nbytes <= self.nbytes
        _ck(rt().cudaMemcpy(self.ptr, arr.ctypes.data_as(C.c_void_p), arr.nbytes, 1), "cudaMemcpy H2D")

    def download(self, arr) -> None:
        assert arr.nbytes <= self.nbytes
        _ck(rt().cudaMemcpy(arr.ctypes.data_as(C.c_void_p), self.ptr, arr.nbytes, 2), "cudaMemcpy D2H")

    def fill(self, byte: int) -> None:
        _ck(rt().cudaMemset(self.ptr, byte, self.nbytes), "cudaMemset")

    def free(self) -> None:
        if self.ptr:
            rt().cudaFree(self.ptr)
            self.ptr = C.c_void_p()


def synchronize() -> None:
    _ck(rt().cudaDeviceSynchronize(), "cudaDeviceSynchronize")


def mem_get_info() -> tuple[int, int]:
    """(free, total) bytes of the current device."""
    free, total = C.c_size_t(), C.c_size_t()
    _ck(rt().cudaMemGetInfo(C.byref(free), C.byref(total)), "cudaMemGetInfo")
    return int(free.value), int(total.value)
