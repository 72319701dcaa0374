"""Python mirror of libvmp's serving API (vmp_server_*, vmp_submit, vmp_poll).

    srv = Server(hbm_budget_bytes=150e9, max_streams=64, workers=32)
    sid = srv.open_stream(abi.default_config(...))     # VmpError(ADMISSION_DENIED) over budget
    srv.submit(sid, package, cookie)                   # returns at once
    for r in srv.poll(timeout_ms=100): ...             # vmp_server_result (cookie, stream, status, result)

Every package runs on the GPU inside libvmp; nothing here computes.
"""
import ctypes as C

from . import abi
from ._lib import VmpError, load
from .lio import LIOBuilder


class Server:
    def __init__(self, hbm_budget_bytes=150e9, max_streams=64, workers=32, queue_depth=64, autotune=True,
                 merge_grid_divisor=16, seg_grid_blocks=152):
        self.lib = load()
        cfg = abi.vmp_server_config()
        self.lib.vmp_server_config_default(C.byref(cfg))
        cfg.hbm_budget_bytes = int(hbm_budget_bytes)
        cfg.max_streams = int(max_streams)
        cfg.workers = int(workers)
        cfg.queue_depth = int(queue_depth)
        cfg.autotune = 1 if autotune else 0
        cfg.merge_grid_divisor = int(merge_grid_divisor)
        cfg.seg_grid_blocks = int(seg_grid_blocks)
        h = C.c_void_p()
        code = self.lib.vmp_server_create(C.byref(cfg), C.byref(h))
        if code != abi.VMP_OK:
            raise VmpError(code, "vmp_server_create")
        self.h = h
        self._cfgs = {}

    def _check(self, code, what):
        if code != abi.VMP_OK:
            msg = (self.lib.vmp_server_last_error(self.h) or b"").decode()
            raise VmpError(code, f"{what}: {msg}")

    def open_stream(self, config):
        sid = C.c_int(-1)
        self._check(self.lib.vmp_server_open_stream(self.h, C.byref(config), C.byref(sid)), "open_stream")
        self._cfgs[sid.value] = config
        return sid.value

    def open_stream_wait(self, config, timeout_ms=-1):
        """open_stream that waits for a slot and budget (vmp_server_open_stream_wait)."""
        sid = C.c_int(-1)
        self._check(self.lib.vmp_server_open_stream_wait(self.h, C.byref(config), int(timeout_ms), C.byref(sid)),
                    "open_stream_wait")
        self._cfgs[sid.value] = config
        return sid.value

    def close_stream(self, sid):
        self._check(self.lib.vmp_server_close_stream(self.h, int(sid)), "close_stream")
        self._cfgs.pop(sid, None)

    def submit(self, sid, pkg, cookie=0):
        scan = pkg.scan()
        self._check(self.lib.vmp_submit(self.h, int(sid), C.byref(scan), pkg.imus, pkg.n_imu, int(cookie)), "submit")

    def submit_livox(self, sid, livox, t_start, imus, n_imu, filter_num=1, range_min=0.5, range_max=20.0, cookie=0):
        """A raw Livox message (numpy array of abi.livox_dtype()) as the
        package: decoded on the device by the worker, the scan's end time
        taken from its last kept point (vmp_submit_livox)."""
        import numpy as np
        livox = np.ascontiguousarray(livox, dtype=abi.livox_dtype())
        self._check(self.lib.vmp_submit_livox(self.h, int(sid), C.c_void_p(livox.ctypes.data), len(livox),
                                              int(filter_num), float(range_min), float(range_max), float(t_start),
                                              imus, int(n_imu), int(cookie)), "submit_livox")

    def submit_device(self, sid, d_pts, n, t_start, t_end, d_imus, n_imu, cookie=0):
        """A package already in device memory (pointers stay valid until polled)."""
        self._check(self.lib.vmp_submit_device(self.h, int(sid), C.c_void_p(d_pts), int(n), float(t_start),
                                               float(t_end), C.c_void_p(d_imus), int(n_imu), int(cookie)),
                    "submit_device")

    def poll(self, max_results=256, timeout_ms=100):
        buf = (abi.vmp_server_result * max_results)()
        n = self.lib.vmp_poll(self.h, buf, max_results, int(timeout_ms))
        if n < 0:
            raise VmpError(abi.VMP_ERR_INVALID_ARG, "poll")
        out = []
        for i in range(n):
            r = abi.vmp_server_result()
            C.pointer(r)[0] = buf[i]
            out.append(r)
        return out

    def stream(self, sid):
        """The stream as a LIOBuilder view (map export, state), once it is idle."""
        h = C.c_void_p()
        self._check(self.lib.vmp_server_stream(self.h, int(sid), C.byref(h)), "stream")
        return LIOBuilder.view(self.lib, h, self._cfgs.get(sid))

    def info(self):
        used, n_open, queued, running = C.c_longlong(), C.c_int(), C.c_int(), C.c_int()
        self._check(self.lib.vmp_server_info(self.h, C.byref(used), C.byref(n_open), C.byref(queued),
                                             C.byref(running)), "info")
        return {"budget_used": used.value, "streams_open": n_open.value, "queued": queued.value,
                "running": running.value}

    def tuning(self):
        """The online autotuner's state (vmp_server_tuning)."""
        d, w, r = C.c_int(), C.c_longlong(), C.c_double()
        self._check(self.lib.vmp_server_tuning(self.h, C.byref(d), C.byref(w), C.byref(r)), "vmp_server_tuning")
        k, b = C.c_int(), C.c_int()
        self._check(self.lib.vmp_server_knob(self.h, b"max_inflight", C.byref(k)), "vmp_server_knob")
        self._check(self.lib.vmp_server_knob(self.h, b"seg_grid_blocks", C.byref(b)), "vmp_server_knob")
        return {"merge_grid_divisor": d.value, "max_inflight": k.value, "seg_grid_blocks": b.value,
                "windows": w.value, "best_rate": r.value}

    def close(self):
        if getattr(self, "h", None):
            self.lib.vmp_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
