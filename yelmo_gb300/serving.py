"""Serving: velocity-solve requests from many ensemble members (ygpu_server_*).

A thin ctypes wrapper of the server in the shared library. The server keeps
every member's state on the device and solves requests with continuous
batching; see ``include/yelmo_gpu.h`` for the contract.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from .gpu import YgpuError, last_error, lib
from .params import YdynParams

FIELDS = {"ux": abi.SRV_UX, "uy": abi.SRV_UY, "visc_eff": abi.SRV_VISC, "H_ice": abi.SRV_H,
          "ux_b": abi.SRV_UXB, "uy_b": abi.SRV_UYB}


class Server:
    """One serving loop on one GPU."""

    def __init__(self, par: YdynParams, device: int = 0, dH_sigma: float = 5.0,
                 hbm_budget: float = 150e9, max_slots: int = 0, max_active_unknowns: int = 0):
        self.L = lib()
        cfg = abi.ServerCfg()
        cfg.device = device
        cfg.kind = par.kind
        cfg.par = par.to_c()
        cfg.grad_lim = par.grad_lim
        cfg.taud_lim = par.taud_lim
        cfg.lateral_bc = abi.LATBC_CODES[par.ssa_lat_bc]
        cfg.dH_sigma = dH_sigma
        cfg.hbm_budget = int(hbm_budget)
        cfg.max_slots = max_slots
        cfg.max_active_unknowns = max_active_unknowns
        self.par = par
        self.srv = self.L.ygpu_server_create(C.byref(cfg))
        if not self.srv:
            raise YgpuError(abi.ERR_CUDA, last_error())
        self.shapes = []

    def close(self):
        if getattr(self, "srv", None):
            self.L.ygpu_server_destroy(self.srv)
            self.srv = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_member(self, state: dict, dx: float, n_glen: float = 3.0, dy: float | None = None) -> int:
        """Register a member from host arrays (a calc_velocity_* field dict)."""
        nx, ny = state["H_ice"].shape
        nz = state["zeta_aa"].shape[0]
        f = abi.Fields()
        f.nx, f.ny, f.nz = nx, ny, nz
        f.dx, f.dy, f.n_glen = dx, dx if dy is None else dy, n_glen
        keep = []
        for name, _ in abi.Fields._fields_[6:]:
            a = state.get(name)
            if isinstance(a, np.ndarray):
                a = np.asfortranarray(a)
                keep.append(a)
                setattr(f, name, a.ctypes.data)
        mid = C.c_int(-1)
        st = self.L.ygpu_server_add_member(self.srv, C.byref(f), C.byref(mid))
        if st != 0:
            raise YgpuError(st, last_error())
        self.shapes.append((nx, ny, nz))
        return mid.value

    def submit(self, member: int, seed: int) -> int:
        rid = C.c_int(-1)
        st = self.L.ygpu_server_submit(self.srv, member, C.c_ulonglong(seed), C.byref(rid))
        if st != 0:
            raise YgpuError(st, last_error())
        return rid.value

    def poll(self, rid: int) -> bool:
        return self.L.ygpu_server_poll(self.srv, rid) == 1

    def wait(self, rid: int, timeout: float = -1.0):
        """Returns (status, stats dict, latency in ms)."""
        st = abi.Stats()
        lat = C.c_double(0.0)
        r = self.L.ygpu_server_wait(self.srv, rid, timeout, C.byref(st), C.byref(lat))
        return int(r), st.as_dict(), lat.value

    def fetch(self, member: int, field: str) -> np.ndarray:
        nx, ny, nz = self.shapes[member]
        shape = (nx, ny, nz) if field == "visc_eff" else (nx, ny)
        out = np.zeros(shape, order="F")
        st = self.L.ygpu_server_fetch(self.srv, member, FIELDS[field], out.ctypes.data_as(C.POINTER(C.c_double)))
        if st != 0:
            raise YgpuError(st, last_error())
        return out

    def info(self) -> dict:
        i = abi.ServerInfo()
        self.L.ygpu_server_get_info(self.srv, C.byref(i))
        return {k: getattr(i, k) for k, _ in abi.ServerInfo._fields_}


def member_state(inst) -> dict:
    """Cold-start host state of a member: the instance's fields with the GPU prologue."""
    from . import gpu
    return gpu.prepare(inst)
