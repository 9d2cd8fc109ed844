"""Host API of the GPU initial-condition generator (PyTorch owns the device
buffers and streams; the work runs in libaarambam_gpu.so).

`ICGenerator(cfg, alpha, x0, k, T)` mirrors one run of the reference
executable for a parameter-file dict `cfg` (keys as in
Aarambam/LPT/Basis/read_param.c:25-184): `run(lagr_pos)` performs
displacement_fields() (main.c:149-1532) on float32 [n, 3] Lagrangian
positions resident on the GPU and returns (pos, vel).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from ._lib import AarError, check


def params_from_config(cfg: dict, precision: int = _lib.AAR_FUSED_FP32, mem_limit_bytes: int = 0,
                       noise_fp64: bool = False, nslab: int = 0) -> _lib.Params:
    """C-ABI parameters of a parameter-file dict; a dict with the A_res /
    w_res / phi_res tags is a 2LPTResBasis set.  noise_fp64: the fused form's
    RNG-to-amplitude step in FP64.  nslab: x-slabs of the slab form."""
    res = "A_res" in cfg
    return _lib.Params(
        nmesh=cfg["Nmesh"], nsample=cfg["Nsample"], nmax=cfg["Nmax"], seed=cfg["Seed"], box=cfg["Box"],
        omega=cfg["Omega"], omega_lambda=cfg["OmegaLambda"], hubble_param=cfg["HubbleParam"],
        sigma8=cfg["Sigma8"], primordial_index=cfg["PrimordialIndex"], redshift=cfg["Redshift"], fnl=cfg["Fnl"],
        unit_length_in_cm=cfg["UnitLength_in_cm"], unit_mass_in_g=cfg["UnitMass_in_g"],
        unit_velocity_in_cm_per_s=cfg["UnitVelocity_in_cm_per_s"],
        input_spectrum_unit_length_in_cm=cfg["InputSpectrum_UnitLength_in_cm"],
        fixed_amplitude=cfg["FixedAmplitude"], phase_flip=cfg["PhaseFlip"], sphere_mode=cfg["SphereMode"],
        precision=precision, mem_limit_bytes=mem_limit_bytes,
        variant=_lib.AAR_VARIANT_RESBASIS if res else _lib.AAR_VARIANT_BASIS,
        which_spectrum=cfg.get("WhichSpectrum", 0), a_res=cfg.get("A_res", 0.0), w_res=cfg.get("w_res", 0.0),
        phi_res=cfg.get("phi_res", 0.0), noise_fp64=int(bool(noise_fp64)), nslab=int(nslab))


def _ptr(t: torch.Tensor) -> int:
    """Address of a contiguous tensor the device can address: CUDA memory,
    or page-locked host memory (pin_memory), which kernels read and write
    directly over the host link."""
    if not (t.is_cuda or t.is_pinned()) or not t.is_contiguous():
        raise ValueError("expected a contiguous CUDA or pinned host tensor")
    return t.data_ptr()


def _dptr(a: np.ndarray):
    return np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(C.POINTER(C.c_double))


class ICGenerator:
    """One plan: grid, cosmology, coefficient tables and transfer function."""

    def __init__(self, cfg: dict, alpha: np.ndarray, x0: np.ndarray, k: np.ndarray, T: np.ndarray,
                 precision: str = "fp32", device=None, mem_limit_bytes: int = 0, noise_fp64: bool = False,
                 nslab: int = 8):
        self.L = _lib.load()
        self.cfg = dict(cfg)
        self.N = int(cfg["Nmesh"])
        self.device = torch.device(device if device is not None else "cuda", torch.cuda.current_device()
                                   if device is None else torch.device(device).index or 0)
        # "slab_fp32": the FP32 arithmetic streamed over nslab x-slabs
        # (AAR_SLAB_FP32), for grids whose fused fields do not fit the GPU
        forms = {"fp32": _lib.AAR_FUSED_FP32, "fp64": _lib.AAR_PLAIN_FP64,
                 "fp64_regrouped": _lib.AAR_PLAIN_FP64_REGROUPED, "slab_fp32": _lib.AAR_SLAB_FP32}
        if precision not in forms:
            raise ValueError(f"precision must be one of {sorted(forms)}")
        self.precision = forms[precision]
        prm = params_from_config(cfg, self.precision, mem_limit_bytes, noise_fp64,
                                 nslab if self.precision == _lib.AAR_SLAB_FP32 else 0)
        h = C.c_void_p()
        with torch.cuda.device(self.device):
            rc = self.L.aar_plan_create(C.byref(prm), C.byref(h))
        self.h = h
        if rc != _lib.AAR_OK:
            msg = self.L.aar_last_error(h) if h else b"plan creation failed"
            self.close()
            raise AarError(rc, msg.decode() if msg else "")
        self._alpha = np.ascontiguousarray(alpha, dtype=np.float64)
        self._x0 = np.ascontiguousarray(x0, dtype=np.float64)
        M = self._alpha.shape[0]
        check(self.L, self.h, self.L.aar_set_tables(self.h, _dptr(self._alpha), _dptr(self._x0), M))
        kk = np.ascontiguousarray(k, dtype=np.float64)
        tt = np.ascontiguousarray(T, dtype=np.float64)
        check(self.L, self.h, self.L.aar_set_transfer(self.h, _dptr(kk), _dptr(tt), len(kk)))

    @property
    def plain(self) -> bool:
        """True for the plain FP64 cuFFT forms."""
        return self.precision in (_lib.AAR_PLAIN_FP64, _lib.AAR_PLAIN_FP64_REGROUPED)

    def prepare(self) -> None:
        """Allocate what a run needs now (aar_plan_prepare): the plain forms'
        fields and cuFFT plans are otherwise made by the first run."""
        with torch.cuda.device(self.device):
            check(self.L, self.h, self.L.aar_plan_prepare(self.h))

    def close(self):
        if getattr(self, "h", None):
            self.L.aar_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def scalars(self) -> dict:
        s = _lib.Scalars()
        check(self.L, self.h, self.L.aar_get_scalars(self.h, C.byref(s)))
        return {n: getattr(s, n) for n, _ in _lib.Scalars._fields_}

    @property
    def launches(self) -> int:
        return self.L.aar_last_launch_count(self.h)

    @property
    def device_bytes(self) -> int:
        """Device memory the plan holds (aar_plan_device_bytes)."""
        return int(self.L.aar_plan_device_bytes(self.h))

    @property
    def n_modes(self) -> int:
        return self._alpha.shape[0]

    def set_tables(self, alpha: np.ndarray, x0: np.ndarray = None) -> None:
        """Replace the coefficient tables (no-op when they are unchanged)."""
        alpha = np.ascontiguousarray(alpha, dtype=np.float64)
        x0 = self._x0 if x0 is None else np.ascontiguousarray(x0, dtype=np.float64)
        if alpha.shape == self._alpha.shape and np.array_equal(alpha, self._alpha) and np.array_equal(x0, self._x0):
            return
        self._alpha, self._x0 = alpha, x0
        check(self.L, self.h, self.L.aar_set_tables(self.h, _dptr(self._alpha), _dptr(self._x0), alpha.shape[0]))

    def set_jit(self, mode: int) -> str:
        """Run-time specialised modal row kernel: 0 off, 1 for N >= 256 (the
        default), 2 always.  Returns the status ("on", "off" or the reason
        the generic kernel is used)."""
        check(self.L, self.h, self.L.aar_set_jit(self.h, int(mode)))
        return self.jit_status

    @property
    def jit_status(self) -> str:
        return self.L.aar_jit_status(self.h).decode()

    def autotune(self) -> str:
        """Time the candidate schedules of this plan on its GPU and keep the
        fastest (aar_autotune); returns the per-candidate report.  The plan's
        spectrum and fields are overwritten."""
        buf = C.create_string_buffer(4096)
        with torch.cuda.device(self.device):
            check(self.L, self.h, self.L.aar_autotune(self.h, buf, len(buf), self._stream()))
        return buf.value.decode()

    def set_seed(self, seed: int) -> None:
        check(self.L, self.h, self.L.aar_set_seed(self.h, int(seed)))
        self.cfg["Seed"] = int(seed)

    def _stream(self):
        return C.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    def seedtable(self) -> torch.Tensor:
        out = torch.empty((self.N, self.N), dtype=torch.int32, device=self.device)
        check(self.L, self.h, self.L.aar_seedtable(self.h, _ptr(out), self._stream()))
        return out

    def stage(self, name: str) -> None:
        fn = getattr(self.L, f"aar_stage_{name}")
        check(self.L, self.h, fn(self.h, self._stream()))

    def spectrum(self) -> torch.Tensor:
        """The plan's current potential spectrum, complex64 [N, N, N/2+1]
        (complex128, the total potential of the last run, for the plain
        forms)."""
        dt = torch.complex128 if self.plain else torch.complex64
        out = torch.empty((self.N, self.N, self.N // 2 + 1), dtype=dt, device=self.device)
        check(self.L, self.h, self.L.aar_copy_spectrum(self.h, _ptr(out), self._stream()))
        return out

    def field(self, which: int) -> torch.Tensor:
        """Displacement field `which` (0..2 ZA, 3..5 2LPT before its 1/N^3):
        float32 for the fused form, float64 for the plain forms (after a run)."""
        dt = torch.float64 if self.plain else torch.float32
        out = torch.empty((self.N, self.N, self.N), dtype=dt, device=self.device)
        check(self.L, self.h, self.L.aar_copy_field(self.h, which, _ptr(out), self._stream()))
        return out

    def c2r(self, spec: torch.Tensor) -> torch.Tensor:
        spec = spec.to(torch.complex64).contiguous()
        out = torch.empty((self.N, self.N, self.N), dtype=torch.float32, device=self.device)
        check(self.L, self.h, self.L.aar_c2r(self.h, _ptr(spec), _ptr(out), self._stream()))
        return out

    def r2c(self, real: torch.Tensor) -> torch.Tensor:
        real = real.to(torch.float32).contiguous()
        out = torch.empty((self.N, self.N, self.N // 2 + 1), dtype=torch.complex64, device=self.device)
        check(self.L, self.h, self.L.aar_r2c(self.h, _ptr(real), _ptr(out), self._stream()))
        return out

    def set_modal_partition(self, part: int, nparts: int) -> None:
        """This plan's share of a modal sum split over radial modes
        (aar_set_modal_partition; (0, 1) is the unsplit sum)."""
        check(self.L, self.h, self.L.aar_set_modal_partition(self.h, int(part), int(nparts)))

    def set_spectrum(self, spec: torch.Tensor) -> None:
        """Replace the plan's potential spectrum (complex [N, N, N/2+1])."""
        spec = spec.to(torch.complex64).contiguous()
        check(self.L, self.h, self.L.aar_set_spectrum(self.h, _ptr(spec), self._stream()))

    def readout(self, lagr: torch.Tensor, pos: torch.Tensor = None, vel: torch.Tensor = None):
        lagr = lagr.contiguous()
        pos = torch.empty_like(lagr) if pos is None else pos
        vel = torch.empty_like(lagr) if vel is None else vel
        check(self.L, self.h, self.L.aar_stage_readout(self.h, _ptr(lagr), lagr.shape[0], _ptr(pos), _ptr(vel),
                                                       self._stream()))
        return pos, vel

    def run(self, lagr: torch.Tensor, pos: torch.Tensor = None, vel: torch.Tensor = None):
        """Whole path on device-resident Lagrangian positions float32 [n, 3]."""
        lagr = lagr.contiguous()
        pos = torch.empty_like(lagr) if pos is None else pos
        vel = torch.empty_like(lagr) if vel is None else vel
        check(self.L, self.h, self.L.aar_run(self.h, _ptr(lagr), lagr.shape[0], _ptr(pos), _ptr(vel),
                                             self._stream()))
        return pos, vel

    def run_glass(self, glass: torch.Tensor, glass_box: float, tile: int):
        glass = glass.contiguous()
        n = glass.shape[0] * tile ** 3
        pos = torch.empty((n, 3), dtype=torch.float32, device=self.device)
        vel = torch.empty_like(pos)
        ids = torch.empty((n,), dtype=torch.int32, device=self.device)
        check(self.L, self.h, self.L.aar_run_glass(self.h, _ptr(glass), glass.shape[0], float(glass_box), tile,
                                                   _ptr(pos), _ptr(vel), _ptr(ids), self._stream()))
        return pos, vel, ids

    def run_lattice(self, glass_n: int, glass_box: float, tile: int, pos: torch.Tensor = None,
                    vel: torch.Tensor = None, ids: torch.Tensor = None):
        """Whole path for the regular glass_n^3 lattice glass tiled tile^3
        times (aar_run_lattice): no glass array; pos / vel float32 [n, 3]
        and ids int32 [n] (optional) on the device or in pinned host memory."""
        n = glass_n ** 3 * tile ** 3
        pos = torch.empty((n, 3), dtype=torch.float32, device=self.device) if pos is None else pos
        vel = torch.empty((n, 3), dtype=torch.float32, device=self.device) if vel is None else vel
        check(self.L, self.h, self.L.aar_run_lattice(self.h, int(glass_n), float(glass_box), int(tile), _ptr(pos),
                                                     _ptr(vel), _ptr(ids) if ids is not None else None,
                                                     self._stream()))
        return pos, vel, ids

    def readout_glass(self, glass: torch.Tensor, glass_box: float, tile: int):
        """Read-out stage alone, Lagrangian positions from the tiled glass."""
        glass = glass.contiguous()
        n = glass.shape[0] * tile ** 3
        pos = torch.empty((n, 3), dtype=torch.float32, device=self.device)
        vel = torch.empty_like(pos)
        ids = torch.empty((n,), dtype=torch.int32, device=self.device)
        check(self.L, self.h, self.L.aar_stage_readout_glass(self.h, _ptr(glass), glass.shape[0], float(glass_box),
                                                             tile, _ptr(pos), _ptr(vel), _ptr(ids), self._stream()))
        return pos, vel, ids

    def run_glass_host(self, glass: np.ndarray, glass_box: float, tile: int, ids: bool = True, out=None,
                       wait: bool = True):
        """Host-buffer glass run (aar_run_glass_host[_async]): the glass goes
        in, positions, velocities (and IDs) come back in host arrays `out`
        = (pos, vel, ids or None), allocated when not given.  wait=False
        returns after enqueueing; call wait_host_copies() before reading."""
        glass = np.ascontiguousarray(glass, dtype=np.float32)
        n = glass.shape[0] * tile ** 3
        if out is None:
            out = (np.empty((n, 3), np.float32), np.empty((n, 3), np.float32),
                   np.empty((n,), np.int32) if ids else None)
        pos, vel, idv = out
        self._glass_keep = glass  # the host glass must outlive an asynchronous copy
        fn = self.L.aar_run_glass_host if wait else self.L.aar_run_glass_host_async
        addr = (lambda a: a.data_ptr()) if isinstance(pos, torch.Tensor) else (lambda a: a.ctypes.data)
        with torch.cuda.device(self.device):
            check(self.L, self.h, fn(self.h, glass.ctypes.data, glass.shape[0], float(glass_box), int(tile),
                                     addr(pos), addr(vel), addr(idv) if idv is not None else None,
                                     self._stream()))
        return pos, vel, idv

    def wait_host_copies(self) -> None:
        check(self.L, self.h, self.L.aar_wait_host_copies(self.h))

    def run_host(self, lagr: np.ndarray):
        """The C-ABI host-buffer path: numpy in, numpy out (copies included)."""
        lagr = np.ascontiguousarray(lagr, dtype=np.float32)
        pos = np.empty_like(lagr)
        vel = np.empty_like(lagr)
        check(self.L, self.h, self.L.aar_run_host(self.h, lagr.ctypes.data, lagr.shape[0], pos.ctypes.data,
                                                  vel.ctypes.data, self._stream()))
        return pos, vel


class ICBatch:
    """Several ICGenerator plans (each with its own seed, table and mode
    count, one device) run as one CUDA graph (aar_batch_*): the first run
    captures every realisation as a branch of the graph, later runs replay it
    with a single launch on the current stream."""

    def __init__(self, gens):
        self.gens = list(gens)
        self.L = _lib.load()
        arr = (C.c_void_p * len(self.gens))(*[g.h.value for g in self.gens])
        b = C.c_void_p()
        rc = self.L.aar_batch_create(arr, len(self.gens), C.byref(b))
        if rc != _lib.AAR_OK:
            raise AarError(rc, "aar_batch_create failed (fused plans on one device required)")
        self.b = b
        self.device = self.gens[0].device

    def close(self):
        if getattr(self, "b", None):
            self.L.aar_batch_destroy(self.b)
            self.b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def launches(self) -> int:
        return self.L.aar_batch_launch_count(self.b)

    def run(self, lagrs, poss, vels):
        """One realisation per plan: lagrs[i] float32 [n_i, 3] on the device;
        results are written into poss[i], vels[i]."""
        n = len(self.gens)
        if not (len(lagrs) == len(poss) == len(vels) == n):
            raise ValueError("one Lagrangian/position/velocity array per plan")
        vp = C.c_void_p
        la = (vp * n)(*[_ptr(t) for t in lagrs])
        pa = (vp * n)(*[_ptr(t) for t in poss])
        va = (vp * n)(*[_ptr(t) for t in vels])
        na = (C.c_int64 * n)(*[t.shape[0] for t in lagrs])
        stream = C.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)
        rc = self.L.aar_batch_run(self.b, la, na, pa, va, stream)
        if rc != _lib.AAR_OK:
            msg = self.L.aar_batch_last_error(self.b)
            raise AarError(rc, msg.decode() if msg else "")
