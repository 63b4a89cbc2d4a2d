"""Python mirror of the qmckl `*_device` context API over the C ABI.

`Context` wraps one qmckl_context_device. Method names follow the reference's functions
without the `qmckl_` prefix and `_device` suffix (set_nucleus_num -> qmckl_set_nucleus_num_device),
take numpy arrays or raw device pointers, and raise QmcklError carrying the reference's
exit code on failure. `load_system` calls the setters in the order of the reference's own
tests (tests/test_qmckl_ao.cpp:122-176, tests/test_qmckl_mo.cpp:80-275).
"""
import ctypes
import os

import numpy as np

from . import capi

SUCCESS = 0
INVALID_ARG_2, INVALID_ARG_3, INVALID_ARG_4 = 2, 3, 4
FAILURE, INVALID_CONTEXT, ALLOCATION_FAILED, NOT_PROVIDED, ALREADY_SET = 101, 103, 104, 106, 108
PRECISION_FP64, PRECISION_SPLIT_BF16 = 0, 1
SHARED_EXP_AUTO, SHARED_EXP_OFF, SHARED_EXP_ON = -1, 0, 1


class QmcklError(RuntimeError):
    def __init__(self, code, function, message):
        super().__init__("%s failed with exit code %d (%s): %s" % (function, code, _string_of(code), message))
        self.code = code
        self.function = function
        self.message = message


def _string_of(code):
    return capi.lib().qmckl_string_of_error_device(code).decode()


class DeviceBuffer:
    """A device allocation registered in the context (freed with it)."""

    def __init__(self, ctx, nbytes):
        self.ctx = ctx
        self.nbytes = int(nbytes)
        self.ptr = ctx.L.qmckl_malloc_device(ctx.handle, max(self.nbytes, 1))
        if not self.ptr:
            raise QmcklError(ALLOCATION_FAILED, "qmckl_malloc_device", "allocation of %d bytes failed" % self.nbytes)

    def free(self):
        if self.ptr:
            self.ctx.L.qmckl_free_device(self.ctx.handle, self.ptr)
            self.ptr = None


class Context:
    def __init__(self, device=0, stream=None):
        self.L = capi.lib()
        if stream is None:
            self.handle = self.L.qmckl_context_create_device(int(device))
        else:
            self.handle = self.L.qmckl_context_create_with_stream_device(int(device), ctypes.c_void_p(int(stream)))
        if not self.handle:
            raise QmcklError(INVALID_CONTEXT, "qmckl_context_create_device", "context creation failed")
        self._buffers = {}
        self.point_num = 0  # points of the last set_point

    # ------------------------------------------------------------------ lifetime
    def close(self):
        if self.handle:
            self.L.qmckl_context_destroy_device(self.handle)
            self.handle = 0

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------------ errors
    def error(self):
        code = ctypes.c_int32(0)
        fn = ctypes.create_string_buffer(256)
        msg = ctypes.create_string_buffer(1024)
        self.L.qmckl_get_error_device(self.handle, ctypes.byref(code), fn, 256, msg, 1024)
        return code.value, fn.value.decode(), msg.value.decode()

    def check(self, rc, name):
        if rc != SUCCESS:
            _, fn, msg = self.error()
            raise QmcklError(rc, fn or name, msg)
        return rc

    def call(self, name, *args):
        """Calls qmckl_<name>_device and raises on a non-zero exit code."""
        f = getattr(self.L, "qmckl_%s_device" % name)
        return self.check(f(self.handle, *args), "qmckl_%s_device" % name)

    # ------------------------------------------------------------------ memory
    def upload(self, array, key=None):
        """Copies a numpy array to a registered device buffer; returns the buffer."""
        a = np.ascontiguousarray(array)
        buf = self._buffers.get(key) if key is not None else None
        if buf is None or buf.nbytes < a.nbytes:
            if buf is not None:
                buf.free()
            buf = DeviceBuffer(self, a.nbytes)
            if key is not None:
                self._buffers[key] = buf
        if a.nbytes:
            self.check(self.L.qmckl_memcpy_H2D(self.handle, buf.ptr, a.ctypes.data_as(ctypes.c_void_p), a.nbytes),
                       "qmckl_memcpy_H2D")
        return buf

    def download(self, ptr, shape, dtype=np.float64):
        out = np.empty(shape, dtype=dtype)
        if out.nbytes:
            self.check(self.L.qmckl_memcpy_D2H(self.handle, out.ctypes.data_as(ctypes.c_void_p), ptr, out.nbytes),
                       "qmckl_memcpy_D2H")
        return out

    def buffer(self, key, nbytes):
        buf = self._buffers.get(key)
        if buf is None or buf.nbytes < nbytes:
            if buf is not None:
                buf.free()
            buf = DeviceBuffer(self, nbytes)
            self._buffers[key] = buf
        return buf

    # ------------------------------------------------------------------ system setup
    def set_nucleus(self, s, transp="T"):
        self.call("set_nucleus_num", s.nucl_num)
        coord = s.nucl_coord if transp == "T" else np.ascontiguousarray(s.nucl_coord.T)
        d = self.upload(coord)
        self.call("set_nucleus_coord", transp.encode(), d.ptr, 3 * s.nucl_num)
        d = self.upload(s.charge)
        self.call("set_nucleus_charge", d.ptr, s.nucl_num)

    def set_ao_basis(self, s):
        up = lambda a, dt: self.upload(np.asarray(a, dtype=dt)).ptr
        self.call("set_ao_basis_type", b"G")
        self.call("set_ao_basis_shell_num", s.shell_num)
        self.call("set_ao_basis_prim_num", s.prim_num)
        self.call("set_ao_basis_nucleus_index", up(s.nucleus_index, np.int64), s.nucl_num)
        self.call("set_ao_basis_nucleus_shell_num", up(s.nucleus_shell_num, np.int64), s.nucl_num)
        self.call("set_ao_basis_shell_ang_mom", up(s.shell_ang_mom, np.int32), s.shell_num)
        self.call("set_ao_basis_shell_factor", up(s.shell_factor, np.float64), s.shell_num)
        self.call("set_ao_basis_shell_prim_num", up(s.shell_prim_num, np.int64), s.shell_num)
        self.call("set_ao_basis_shell_prim_index", up(s.shell_prim_index, np.int64), s.shell_num)
        self.call("set_ao_basis_exponent", up(s.exponent, np.float64), s.prim_num)
        self.call("set_ao_basis_coefficient", up(s.coefficient, np.float64), s.prim_num)
        self.call("set_ao_basis_prim_factor", up(s.prim_factor, np.float64), s.prim_num)
        self.call("set_ao_basis_ao_num", s.ao_num)
        self.call("set_ao_basis_ao_factor", up(s.ao_factor, np.float64), s.ao_num)

    def set_mo_basis(self, s):
        self.call("set_mo_basis_mo_num", s.mo_num)
        d = self.upload(s.mo_coef)
        self.call("set_mo_basis_coefficient", d.ptr)

    def read_trexio(self, path):
        """Electrons, nuclei, basis, AOs and MOs from a TREXIO file (qmckl_trexio_read_device;
        libtrexio is loaded at run time, see include/qmckl_gpu.h)."""
        name = os.fsencode(path)
        self.call("trexio_read", name, len(name))

    def set_point(self, coord, transp="N", host=False):
        """coord is [P][3] for 'N' or [3][P] for 'T'. With host=True the host array is
        passed directly (the library copies it); otherwise it is uploaded first."""
        c = np.ascontiguousarray(coord, dtype=np.float64)
        num = c.shape[0] if transp == "N" else c.shape[1]
        ptr = c.ctypes.data_as(ctypes.c_void_p) if host else self.upload(c, key="points").ptr
        self.call("set_point", transp.encode(), num, ptr, 3 * num)
        self.point_num = int(num)

    def load_system(self, s, mo=True, points=True):
        self.set_nucleus(s)
        self.set_ao_basis(s)
        if mo and s.mo_num > 0:
            self.set_mo_basis(s)
        if points:
            self.set_point(s.coord)

    # ------------------------------------------------------------------ results
    def _num(self, getter):
        v = ctypes.c_int64(0)
        self.call(getter, ctypes.byref(v))
        return v.value

    @property
    def ao_num(self):
        return self._num("get_ao_basis_ao_num")

    @property
    def mo_num(self):
        return self._num("get_mo_basis_mo_num")

    def _get(self, name, shape, inplace=False):
        out = np.empty(shape)
        self.call(name + ("_inplace" if inplace else ""), out.ctypes.data_as(ctypes.c_void_p), out.size)
        return out

    def get_ao_vgl(self, point_num, inplace=False):
        return self._get("get_ao_basis_ao_vgl", (point_num, 5, self.ao_num), inplace)

    def get_ao_value(self, point_num, inplace=False):
        return self._get("get_ao_basis_ao_value", (point_num, self.ao_num), inplace)

    def get_shell_vgl(self, point_num, shell_num):
        return self._get("get_ao_basis_shell_vgl", (point_num, 5, shell_num))

    def get_mo_vgl(self, point_num, inplace=False):
        return self._get("get_mo_basis_mo_vgl", (point_num, 5, self.mo_num), inplace)

    def get_mo_value(self, point_num, inplace=False):
        return self._get("get_mo_basis_mo_value", (point_num, self.mo_num), inplace)

    def touch(self):
        self.check(self.L.qmckl_context_touch_device(self.handle), "qmckl_context_touch_device")

    def set_precision(self, mode):
        self.call("set_precision_mode", int(mode))

    def set_shared_exponentials(self, mode):
        self.call("set_ao_shared_exponentials", int(mode))

    def shared_exponentials(self):
        v = ctypes.c_int32(0)
        self.call("get_ao_shared_exponentials", ctypes.byref(v))
        return bool(v.value)

    def vjp_mo_vgl(self, w, want=("coef", "expo", "coord"), prim_num=None):
        """Gradients of sum(w * mo_vgl) (w: [P][5][M] numpy): dict with 'coef' [M][A],
        'expo' [prim_num], 'coord' [P][3] (host arrays passed to the C ABI)."""
        w = np.ascontiguousarray(w, dtype=np.float64)
        P = w.shape[0]
        M, A = self.mo_num, self.ao_num
        K = prim_num if prim_num is not None else self._num("get_ao_basis_prim_num")
        out = {k: None for k in ("coef", "expo", "coord")}
        if "coef" in want:
            out["coef"] = np.empty((M, A))
        if "expo" in want:
            out["expo"] = np.empty(K)
        if "coord" in want:
            out["coord"] = np.empty((P, 3))

        def arg(a):
            return (a.ctypes.data_as(ctypes.c_void_p), a.size) if a is not None else (None, 0)

        self.call("vjp_mo_vgl", w.ctypes.data_as(ctypes.c_void_p), w.size, *arg(out["coef"]), *arg(out["expo"]),
                  *arg(out["coord"]))
        return {k: v for k, v in out.items() if v is not None}

    def vjp_ao_vgl(self, ao_bar, want=("expo", "coord"), prim_num=None):
        ao_bar = np.ascontiguousarray(ao_bar, dtype=np.float64)
        P = ao_bar.shape[0]
        K = prim_num if prim_num is not None else self._num("get_ao_basis_prim_num")
        e = np.empty(K) if "expo" in want else None
        c = np.empty((P, 3)) if "coord" in want else None
        self.call("vjp_ao_vgl", ao_bar.ctypes.data_as(ctypes.c_void_p), ao_bar.size,
                  e.ctypes.data_as(ctypes.c_void_p) if e is not None else None, 0 if e is None else e.size,
                  c.ctypes.data_as(ctypes.c_void_p) if c is not None else None, 0 if c is None else c.size)
        return {k: v for k, v in (("expo", e), ("coord", c)) if v is not None}

    # ------------------------------------------------------------------ GB300 extensions
    def set_async(self, on):
        self.call("set_async", 1 if on else 0)

    def synchronize(self):
        self.check(self.L.qmckl_synchronize_device(self.handle), "qmckl_synchronize_device")

    @property
    def stream(self):
        return self.L.qmckl_get_stream_device(self.handle)

    def set_profiling(self, on):
        self.call("set_profiling", 1 if on else 0)

    def reset_kernel_stats(self):
        self.call("reset_kernel_stats")

    def kernel_stats(self):
        """{kernel name: (launches, total_ms)} for the kernels this context launched."""
        n = self.L.qmckl_get_kernel_stats_device(self.handle, -1, None, 0, None, None)
        out = {}
        for i in range(max(n, 0)):
            name = ctypes.create_string_buffer(128)
            launches = ctypes.c_int64(0)
            ms = ctypes.c_double(0)
            self.L.qmckl_get_kernel_stats_device(self.handle, i, name, 128, ctypes.byref(launches), ctypes.byref(ms))
            out[name.value.decode()] = (launches.value, ms.value)
        return out

    def launch_count(self):
        return self.L.qmckl_get_launch_count_device(self.handle)


class Batch:
    """Several member contexts evaluated together (qmckl_batch_*_device): one persistent launch
    per stage over every member, replayed as a CUDA graph. Results land in the members' caches,
    so `member.get_mo_vgl(P)` reads them afterwards."""

    def __init__(self, members):
        self.L = capi.lib()
        self.members = list(members)
        handles = (ctypes.c_int64 * len(self.members))(*[m.handle for m in self.members])
        self.handle = self.L.qmckl_batch_create_device(handles, len(self.members))
        if not self.handle:
            raise QmcklError(INVALID_CONTEXT, "qmckl_batch_create_device", "batch creation failed")

    def close(self):
        if self.handle:
            self.L.qmckl_batch_destroy_device(self.handle)
            self.handle = 0

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def call(self, name, *args):
        rc = getattr(self.L, "qmckl_batch_%s_device" % name)(self.handle, *args)
        return self.members[0].check(rc, "qmckl_batch_%s_device" % name)

    def set_precision(self, mode):
        self.call("set_precision_mode", int(mode))

    def set_graph(self, on):
        self.call("set_graph", 1 if on else 0)

    def set_async(self, on):
        self.call("set_async", 1 if on else 0)

    def synchronize(self):
        self.call("synchronize")

    def touch(self):
        self.call("touch")

    def provide_mo_vgl(self):
        self.call("provide_mo_vgl")

    def autotune(self):
        self.call("autotune")

    def tuning(self):
        p = (ctypes.c_int32 * 3)()
        self.call("get_tuning", p, 3)
        return tuple(p)

    def set_tuning(self, params):
        p = (ctypes.c_int32 * 3)(*[int(x) for x in params])
        self.call("set_tuning", p, 3)

    def launch_count(self):
        return self.L.qmckl_batch_get_launch_count_device(self.handle)

    def get_mo_vgl(self):
        """[member] -> numpy [P][5][M] (provides first)."""
        self.provide_mo_vgl()
        return [m.get_mo_vgl(m.point_num) for m in self.members]
