"""Serving: continuous batching of simulation requests over resident scenes
(hsr_server_* in include/hsr_gb300.h).

    srv = Server(flags=tracer, max_slots=64)
    sid = srv.add_scene(backend)                    # a gb300.Backend (its scene stays resident)
    req = srv.submit(sid, rf, 256, tx, rx, 1 << 20)  # returns at once
    row, info = req.result()                        # complex64[N], timing of the request

Each request's row equals the row gb300.Backend.simulate_batch gives for the same pose,
chirp, budget and index offset (same Halton samples; only the summation order differs).
"""
import ctypes

import numpy as np

from . import _lib


class Request:
    """A submitted request: result() blocks until its row is written."""

    def __init__(self, server, ticket, row):
        self._server = server
        self.ticket = ticket
        self._row = row  # keeps the output buffer alive until completion
        self._info = None

    def done(self):
        if self._info is None:
            self._wait(0)
        return self._info is not None

    def _wait(self, timeout_ms):
        res = _lib.RequestResultC()
        st = _lib.lib().hsr_server_wait(self._server._h, ctypes.c_uint64(self.ticket), int(timeout_ms),
                                        ctypes.byref(res))
        if st == _lib.HSR_ERR_TIMEOUT:
            return False
        _lib.check(st)
        self._server._pending.pop(self.ticket, None)
        self._info = {"status": res.status, "ticks": res.ticks, "queue_ms": res.queue_ms,
                      "latency_ms": res.latency_ms}
        return True

    def result(self, timeout=None):
        """(row, info): the fetchFrame row and {status, ticks, queue_ms, latency_ms}.
        Raises HsrError if the request failed, TimeoutError if `timeout` (s) passes."""
        if self._info is None:
            if not self._wait(-1 if timeout is None else int(timeout * 1000)):
                raise TimeoutError("request %d still running" % self.ticket)
        if self._info["status"] != _lib.HSR_OK:
            raise _lib.HsrError(self._info["status"], "served request failed")
        return self._row, dict(self._info)


class Server:
    """A request loop on one GPU: resident scenes, admission by slots and device memory,
    batching ticks over every admitted request (see hsr_serve.cu)."""

    def __init__(self, flags=None, phase_mode=_lib.HSR_PHASE_REFERENCE_FP32, max_slots=None,
                 max_samples_per_chirp=None, memory_bytes=None, tick_ms=None):
        L = _lib.lib()
        cfg = _lib.ServerConfigC()
        L.hsr_default_server_config(ctypes.byref(cfg))
        if flags is not None:
            cfg.flags = flags.flags_c() if hasattr(flags, "flags_c") else flags
        cfg.phase_mode = int(phase_mode)
        if max_slots is not None:
            cfg.max_slots = int(max_slots)
        if max_samples_per_chirp is not None:
            cfg.max_samples_per_chirp = int(max_samples_per_chirp)
        if memory_bytes is not None:
            cfg.memory_bytes = int(memory_bytes)
        if tick_ms is not None:
            cfg.tick_ms = float(tick_ms)
        h = ctypes.c_void_p()
        _lib.check(L.hsr_server_create(ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h
        self._scenes = []  # keeps the backends (and their device scenes) alive
        # requests whose row the worker may still write (the C ABI needs out_row valid
        # until completion, even if the caller drops the handle)
        self._pending = {}

    def add_scene(self, backend):
        sid = ctypes.c_int32()
        _lib.check(_lib.lib().hsr_server_add_scene(self._h, backend.handle, ctypes.byref(sid)))
        self._scenes.append(backend)
        return sid.value

    def submit(self, scene, rf, samples_per_chirp, tx, rx, budget, index_offset=0):
        row = np.zeros(int(samples_per_chirp), np.complex64)
        r = _lib.RequestC()
        r.scene = int(scene)
        r.samples_per_chirp = int(samples_per_chirp)
        r.rf = rf.to_c()
        r.tx = tx.to_c()
        r.rx = rx.to_c()
        r.budget = int(budget)
        r.index_offset = int(index_offset)
        r.out_row = row.ctypes.data
        t = ctypes.c_uint64()
        _lib.check(_lib.lib().hsr_server_submit(self._h, ctypes.byref(r), ctypes.byref(t)))
        req = Request(self, t.value, row)
        self._pending[t.value] = req
        return req

    def stats(self):
        s = _lib.ServerStatsC()
        _lib.check(_lib.lib().hsr_server_get_stats(self._h, ctypes.byref(s)))
        return {name: getattr(s, name) for name, _ in _lib.ServerStatsC._fields_}

    def reset_stats(self):
        _lib.check(_lib.lib().hsr_server_reset_stats(self._h))

    def close(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            _lib.lib().hsr_server_destroy(h)  # finishes the ticks on the device first
            self._h = None
            self._pending.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def plan_tick(remaining, target, tile=4096):
    """The server's tick planner (host only): chunk per request."""
    rem = np.ascontiguousarray(remaining, np.int64)
    out = np.zeros(len(rem), np.int64)
    _lib.check(_lib.lib().hsr_debug_plan_tick(len(rem), _lib.ptr(rem), int(target), int(tile), _lib.ptr(out)))
    return out
