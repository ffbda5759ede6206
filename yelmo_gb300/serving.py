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
          "ux_b": abi.SRV_UXB, "uy_b": abi.SRV_UYB, "taub_acx": abi.SRV_TAUBX, "taub_acy": abi.SRV_TAUBY,
          "beta": abi.SRV_BETA, "beta_acx": abi.SRV_BETAX, "beta_acy": abi.SRV_BETAY}
# the member fields a checkpoint holds (with the step count)
CHECKPOINT_FIELDS = ("H_ice", "ux", "uy", "ux_b", "uy_b", "visc_eff", "taub_acx", "taub_acy",
                     "beta", "beta_acx", "beta_acy")


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
        if field not in FIELDS:
            raise ValueError(f"unknown member field {field!r}")
        out = np.zeros(shape, order="F")
        st = self.L.ygpu_server_fetch(self.srv, member, FIELDS[field], out.ctypes.data_as(C.POINTER(C.c_double)))
        if st != 0:
            raise YgpuError(st, last_error())
        return out

    def steps(self, member: int) -> int:
        """Requests of the member admitted so far (the index of its next step)."""
        n = C.c_ulonglong(0)
        st = self.L.ygpu_server_member_steps(self.srv, member, C.byref(n))
        if st != 0:
            raise YgpuError(st, last_error())
        return int(n.value)

    def checkpoint(self, member: int) -> dict:
        """The member's evolving state (an idle member): CHECKPOINT_FIELDS and its
        step count. With the member's fixed inputs it is everything restore() needs;
        np.savez of the dict is a restart file."""
        ck = {k: self.fetch(member, k) for k in CHECKPOINT_FIELDS}
        ck["steps"] = np.int64(self.steps(member))
        return ck

    def restore(self, fixed: dict, ck: dict, dx: float, n_glen: float = 3.0) -> int:
        """Register a member from a checkpoint and its fixed inputs (z_bed, z_sl,
        c_bed, f_slide, ATT, zeta_aa); members restored in their original order keep
        their ids, so their next requests solve what the uninterrupted server would."""
        kind_diva = self.par.kind == abi.KIND_DIVA
        state = {k: fixed[k] for k in ("z_bed", "z_sl", "c_bed", "f_slide", "ATT", "zeta_aa")}
        for k in CHECKPOINT_FIELDS:
            if k in ("ux", "uy"):
                state[(k + "_bar") if kind_diva else (k + "_b")] = ck[k]
            else:
                state[k] = ck[k]
        m = self.add_member(state, dx, n_glen)
        st = self.L.ygpu_server_set_member_steps(self.srv, m, C.c_ulonglong(int(ck["steps"])))
        if st != 0:
            raise YgpuError(st, last_error())
        return m

    def info(self) -> dict:
        i = abi.ServerInfo()
        self.L.ygpu_server_get_info(self.srv, C.byref(i))
        return {k: getattr(i, k) for k, _ in abi.ServerInfo._fields_}


def member_state(inst) -> dict:
    """Cold-start host state of a member: the instance's fields with the GPU prologue."""
    from . import gpu
    return gpu.prepare(inst)
