"""Device handle and device tensors for the host-side API.

A ``DeviceTensor`` is a block of libfmpt device memory holding one tensor in
the reference's column-major layout (Julia storage order of the TensorKit
tensor), real float64 or complex128 as split real/imaginary planes.
"""

import ctypes

import numpy as np

from ._native import C128, F64, FMPTError, check, lib

__all__ = ["Handle", "default_handle", "DeviceTensor", "to_host_mpo"]


class Handle:
    """Owns one fmpt_handle (CUDA stream, cuSOLVER handle, memory pool)."""

    def __init__(self, device=0):
        h = ctypes.c_void_p()
        st = lib().fmpt_create(int(device), ctypes.byref(h))
        if st != 0:
            raise FMPTError(st, "fmpt_create(%d) failed: is a CUDA GPU visible?" % device)
        self.ptr = h
        self.device = device

    def synchronize(self):
        check(lib().fmpt_synchronize(self.ptr), self.ptr)

    def set_svd_method(self, method="gesvd"):
        """SVD routine of the truncated splits: "gesvd" (default), "gesvdp"
        (polar decomposition) or "gesvdj" (one-sided Jacobi)."""
        codes = {"gesvd": 0, "gesvdp": 1, "gesvdj": 2}
        if method not in codes:
            raise ValueError("svd method must be 'gesvd', 'gesvdp' or 'gesvdj'")
        self.check(lib().fmpt_set_svd_method(self.ptr, codes[method]))

    def set_tc_tile(self, tile="pair"):
        """Tile of the tensor-core GEMMs: "pair" (default; 256x256 on two-CTA clusters
        where the GEMM has more than 128 rows) or "single" (one CTA per tile)."""
        codes = {"pair": 0, "single": 1}
        if tile not in codes:
            raise ValueError("tc tile must be 'pair' or 'single'")
        self.check(lib().fmpt_set_tc_tile(self.ptr, codes[tile]))

    def set_f64_engine(self, engine="cuda_cores"):
        """Engine of this handle's FP64 GEMMs: "cuda_cores" (default) or "tensor_cores"
        (the Ozaki-scheme FP64 GEMM on the BF16 tensor cores wherever it is faster)."""
        codes = {"cuda_cores": 0, "tensor_cores": 1}
        if engine not in codes:
            raise ValueError("f64 engine must be 'cuda_cores' or 'tensor_cores'")
        self.check(lib().fmpt_set_f64_engine(self.ptr, codes[engine]))

    def set_wait_test(self, timeout_s=0.0, hold=False):
        """Failure-detection test hook: bound of the grid-barrier waits of the grouped
        kernel and of the fused Krylov step (0: the default 2 s); hold=True makes them
        wait for an arrival that never comes."""
        self.check(lib().fmpt_set_wait_test(self.ptr, int(timeout_s * 1e9), 1 if hold else 0))

    def set_graphs(self, on=True):
        """CUDA-graph Krylov solves for block-sparse operators (default on)."""
        self.check(lib().fmpt_set_graphs(self.ptr, 1 if on else 0))

    def set_fused_krylov(self, on=True):
        """One cooperative launch per Arnoldi orthogonalisation step of the Krylov
        exponentials (default on); off: seven launches, bit-identical results."""
        self.check(lib().fmpt_set_fused_krylov(self.ptr, 1 if on else 0))

    def set_cluster_qr(self, on=True):
        """Thin QR of small tall panels on one thread-block cluster (default on); off:
        cuSOLVER geqrf + ungqr.  Same LAPACK conventions either way."""
        self.check(lib().fmpt_set_cluster_qr(self.ptr, 1 if on else 0))

    def graph_count(self):
        return int(lib().fmpt_graph_launch_count(self.ptr))

    def set_tuning(self, mode=0):
        """Grouped-kernel variant choice: 0 autotune over tiles and block schedules (default),
        1 / 2 force 32x32 / 64x64 tiles with the blocks-by-work schedule, 3 / 4 the same tiles
        with the tiles-by-work schedule."""
        self.check(lib().fmpt_set_tuning(self.ptr, int(mode)))

    def tuning_info(self):
        n, t = ctypes.c_int(), ctypes.c_int64()
        self.check(lib().fmpt_tuning_info(self.ptr, ctypes.byref(n), ctypes.byref(t)))
        return n.value, t.value

    def launch_count(self):
        return int(lib().fmpt_launch_count(self.ptr))

    def profile(self, on=True):
        """Enable/disable the per-kernel-class device timers."""
        check(lib().fmpt_profile_enable(self.ptr, 1 if on else 0), self.ptr)

    def profile_read(self, kernel_class):
        """(launches, device ms) of one class since the last read
        (0 tensor-core GEMM, 1 FP64 GEMM, 2 MPO step, 3 conversion)."""
        n = ctypes.c_int64()
        ms = ctypes.c_double()
        check(lib().fmpt_profile_read(self.ptr, int(kernel_class), ctypes.byref(n),
                                      ctypes.byref(ms)), self.ptr)
        return n.value, ms.value

    def set_stream(self, stream_ptr):
        check(lib().fmpt_set_stream(self.ptr, ctypes.c_void_p(stream_ptr)), self.ptr)

    def check(self, status):
        return check(status, self.ptr)

    def close(self):
        if self.ptr:
            lib().fmpt_destroy(self.ptr)
            self.ptr = None


_default = None


def default_handle():
    global _default
    if _default is None:
        _default = Handle(0)
    return _default


def _dtype_code(dt):
    return C128 if np.issubdtype(np.dtype(dt), np.complexfloating) else F64


class DeviceTensor:
    """A tensor in device memory; ``shape`` uses the reference's index order."""

    __slots__ = ("h", "shape", "dtype", "ptr", "capacity", "__weakref__")

    def __init__(self, shape, dtype=np.float64, handle=None, zero=False):
        self.h = handle or default_handle()
        self.shape = tuple(int(s) for s in shape)
        self.dtype = np.dtype(np.complex128 if _dtype_code(dtype) == C128 else np.float64)
        self.capacity = self.nbytes
        p = ctypes.c_void_p()
        self.h.check(lib().fmpt_malloc(self.h.ptr, self.capacity, ctypes.byref(p)))
        self.ptr = p.value or 0
        if zero:
            self.h.check(lib().fmpt_memset_zero(self.h.ptr, self.ptr, self.nbytes))

    @property
    def code(self):
        return C128 if self.dtype == np.complex128 else F64

    @property
    def nbytes(self):
        n = int(np.prod(self.shape)) if self.shape else 1
        return n * 8 * (2 if self.code == C128 else 1)

    @property
    def size(self):
        return int(np.prod(self.shape)) if self.shape else 1

    def __del__(self):
        try:
            if self.ptr and self.h.ptr:
                lib().fmpt_free(self.h.ptr, self.ptr)
        except Exception:
            pass
        self.ptr = 0

    @staticmethod
    def from_numpy(arr, handle=None, dtype=None):
        arr = np.asarray(arr)
        dt = dtype or (np.complex128 if np.iscomplexobj(arr) else np.float64)
        t = DeviceTensor(arr.shape, dt, handle)
        host = to_host_buffer(arr, t.dtype)
        t.h.check(lib().fmpt_memcpy_h2d(t.h.ptr, t.ptr, host.ctypes.data, t.nbytes))
        t.h.synchronize()
        return t

    def numpy(self):
        n = self.size
        if self.code == C128:
            buf = np.empty(2 * n, dtype=np.float64)
        else:
            buf = np.empty(n, dtype=np.float64)
        self.h.check(lib().fmpt_memcpy_d2h(self.h.ptr, buf.ctypes.data, self.ptr, self.nbytes))
        if self.code == C128:
            flat = buf[:n] + 1j * buf[n:]
        else:
            flat = buf
        return flat.reshape(self.shape, order="F")

    def copy(self):
        t = DeviceTensor(self.shape, self.dtype, self.h)
        self.h.check(lib().fmpt_memcpy_d2d(self.h.ptr, t.ptr, self.ptr, self.nbytes))
        return t

    def reshape(self, shape):
        """A new tensor sharing nothing: column-major reshape (a device copy)."""
        if int(np.prod(shape)) != self.size:
            raise ValueError("DimensionMismatch: reshape %s -> %s" % (self.shape, shape))
        t = self.copy()
        t.shape = tuple(shape)
        return t

    def view_as(self, shape):
        """Reinterpret the same memory with another column-major shape."""
        n = int(np.prod(shape))
        if n * 8 * (2 if self.code == C128 else 1) > self.capacity:
            raise ValueError("DimensionMismatch: view %s -> %s" % (self.shape, shape))
        self.shape = tuple(int(s) for s in shape)
        return self

    def __repr__(self):
        return "DeviceTensor(shape=%s, dtype=%s)" % (self.shape, self.dtype)


def to_host_buffer(arr, dtype):
    """Column-major float64 buffer; complex as split planes (re then im)."""
    arr = np.asarray(arr)
    flat = arr.reshape(-1, order="F")
    if np.dtype(dtype) == np.complex128:
        flat = flat.astype(np.complex128)
        return np.ascontiguousarray(np.concatenate([flat.real, flat.imag]))
    if np.iscomplexobj(flat):
        if np.any(flat.imag != 0):
            raise TypeError("complex data for a real tensor")
        flat = flat.real
    return np.ascontiguousarray(flat.astype(np.float64))


def to_host_mpo(W, dtype):
    """Host buffer of a dense MPO tensor W[wl, s_out, wr, s_in] for the C ABI."""
    return to_host_buffer(W, dtype)
