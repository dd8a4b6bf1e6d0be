"""GB300 3D space-charge kick with Ocelot's ``SpaceCharge`` plugin surface.

``SpaceCharge`` keeps the constructor, attributes and hooks of Ocelot's
``SpaceCharge`` physics process (ocelot/cpbd/sc.py:76-258) so that it drops
into ``Navigator.add_physics_proc`` and ``track()`` unchanged; the numerical
body runs in libocelot_sc (sm_103a CUDA) through its C ABI, with PyTorch
tensors as device storage.  There is no CPU fallback.

Two forms (constructor keyword ``precision``):

* ``"fp64"`` (default, the plain form): FP64 end to end; reproduces the
  reference's ``apply`` to ~1e-10 relative on ``rparticles``.
* ``"fp32"`` (the precision form): FP32 deposit, FFT convolution (field
  differences in Fourier space) and gather, FP64 Green's-function table and
  FP64 accumulation of the kick into ``rparticles``.

``apply(p_array, zstep)`` accepts Ocelot's host ``ParticleArray`` (numpy
arrays; copied to the GPU and back each call, like the reference mutating
``p_array.rparticles`` in place) or a ``DeviceParticleArray`` whose tensors
already live on the GPU (no copies, no host synchronisation).
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _native as N
from .physics_proc import PhysProc

_PREC = {"fp64": N.SC_FP64, "fp32": N.SC_FP32}


def plan_mode(precision: str, deposit: str = "fixed", igf: str = "hybrid", fields: str = "spectral") -> int:
    """Mode bits of a plan (include/ocelot_sc.h): the FP32 form's options."""
    if precision not in _PREC:
        raise ValueError(f"precision must be one of {sorted(_PREC)}, not {precision!r}")
    if deposit not in ("fixed", "sorted"):
        raise ValueError(f"deposit must be 'fixed' or 'sorted', not {deposit!r}")
    if igf not in ("hybrid", "exact"):
        raise ValueError(f"igf must be 'hybrid' or 'exact', not {igf!r}")
    if fields not in ("difference", "spectral"):
        raise ValueError(f"fields must be 'difference' or 'spectral', not {fields!r}")
    mode = _PREC[precision]
    if precision == "fp32":
        if deposit == "sorted":
            mode |= N.SC_FP32_SORTED_DEPOSIT
        if igf == "exact":
            mode |= N.SC_FP32_EXACT_IGF
        if fields == "spectral":
            mode |= N.SC_FP32_SPECTRAL_FIELDS
    return mode


def _torch():
    import torch
    return torch


def cuda_device(device=None):
    """``device`` as a CUDA device with its index ("cuda" is the current device)."""
    torch = _torch()
    d = torch.device(device) if device is not None else torch.device("cuda")
    if d.type != "cuda":
        raise ValueError(f"{d}: the kick runs on a CUDA device")
    return d if d.index is not None else torch.device("cuda", torch.cuda.current_device())


def check_beam_tensors(rp, q, n: int, device):
    """The kernels read n particles of rparticles [6, >= n] (contiguous rows)
    and n charges from q: both float64 tensors on ``device``.  Raises before
    anything is launched when that does not hold."""
    torch = _torch()
    if not (isinstance(rp, torch.Tensor) and isinstance(q, torch.Tensor)):
        raise TypeError("rparticles and q_array must be torch tensors")
    if rp.dtype != torch.float64 or q.dtype != torch.float64:
        raise TypeError(f"rparticles and q_array must be float64, not {rp.dtype} / {q.dtype}")
    if rp.device != device or q.device != device:
        raise ValueError(f"rparticles ({rp.device}) and q_array ({q.device}) must be on {device}")
    if rp.dim() != 2 or rp.shape[0] != 6 or rp.shape[1] < n:
        raise ValueError(f"rparticles must have shape (6, N) with N >= {n}, not {tuple(rp.shape)}")
    if rp.stride(1) != 1:
        raise ValueError("rparticles rows must be contiguous")
    if q.dim() != 1 or q.numel() < n or not q.is_contiguous():
        raise ValueError(f"q_array must be a contiguous vector of {n} charges, not {tuple(q.shape)}")


def _ptr(t) -> C.c_void_p:
    return C.c_void_p(t.data_ptr())


def _stream(device) -> C.c_void_p:
    torch = _torch()
    return C.c_void_p(torch.cuda.current_stream(device).cuda_stream)


class Engine:
    """A plan (mesh shape, precision) and its device workspace on one GPU."""

    def __init__(self, shape, precision: str, device=None, mode=None, tuned: bool = True):
        torch = _torch()
        if not torch.cuda.is_available():
            raise N.NativeLibraryError("ocelot_gb300 needs a CUDA device; there is no CPU fallback")
        self.lib = N.lib()
        self.device = cuda_device(device)
        self.shape = tuple(int(v) for v in shape)
        self.precision = precision
        self.mode = plan_mode(precision) if mode is None else int(mode)
        plan = C.c_void_p()
        with torch.cuda.device(self.device):
            N.check(self.lib.sc_plan_create(C.byref(plan), *self.shape, self.mode))
        self.plan = plan
        self.ws = None
        self.cap = -1
        # launch shapes from the autotuner's table (ocelot_gb300/tuning.py),
        # applied per particle count; tuned=False keeps the plan's defaults
        self.tuned = bool(tuned)
        self._tuned_n = None
        self._rp = None
        self._q = None

    def __del__(self):
        try:
            if getattr(self, "plan", None) is not None and self.plan.value:
                self.lib.sc_plan_destroy(self.plan)
        except Exception:
            pass

    def fft_shape(self):
        m = [C.c_int(), C.c_int(), C.c_int()]
        N.check(self.lib.sc_plan_fft_shape(self.plan, *[C.byref(v) for v in m]))
        return tuple(v.value for v in m)

    def ensure(self, n: int):
        """Grow the workspace to hold kicks of n particles."""
        torch = _torch()
        if n <= self.cap:
            return
        cap = max(n, int(self.cap * 1.25) if self.cap > 0 else n)
        nbytes = int(self.lib.sc_workspace_bytes(self.plan, cap))
        if nbytes < 0:
            raise ValueError(f"bad particle count {n}")
        self.ws = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
        with torch.cuda.device(self.device):
            N.check(self.lib.sc_workspace_init(self.plan, _ptr(self.ws), nbytes, _stream(self.device)))
        self.cap = cap

    def staging(self, n: int):
        torch = _torch()
        if self._rp is None or self._rp.shape[1] < n:
            # even row stride: the kernels then move rows with 16-byte accesses
            self._rp = torch.empty((6, n + (n & 1)), dtype=torch.float64, device=self.device)
            self._q = torch.empty(n, dtype=torch.float64, device=self.device)
        return self._rp[:, :n], self._q[:n]

    def kick(self, rp, q, n: int, energy_gev: float, zstep: float, mesh_scale=math.nan, mesh_shift=math.nan):
        """Launch one kick on the current stream (asynchronous)."""
        torch = _torch()
        check_beam_tensors(rp, q, n, self.device)
        self.ensure(n)
        self.apply_tuning(n)
        ld = rp.stride(0)
        with torch.cuda.device(self.device):
            N.check(self.lib.sc_kick(self.plan, _ptr(self.ws), self.ws.numel(), _ptr(rp), ld, _ptr(q), n,
                                     float(energy_gev), float(zstep), float(mesh_scale), float(mesh_shift),
                                     _stream(self.device)))

    def region(self, name: str, n: int | None = None):
        """A view of an intermediate of the last call (charge grid, potential,
        field grids [nx][ny][nz]; keys [n]; the status ints "status" and
        "first_error", one element each; "field" [3, nX], the field at each
        particle of the last kick when SC_PARAM_RECORD_FIELD is set)."""
        torch = _torch()
        off, nb = C.c_int64(), C.c_int64()
        N.check(self.lib.sc_workspace_region(self.plan, max(self.cap, 0), N.REGIONS[name], C.byref(off), C.byref(nb)))
        raw = self.ws[off.value:off.value + nb.value]
        if name in ("keys", "status", "first_error"):
            return raw.view(torch.int32)
        dt = torch.float64 if self.precision == "fp64" else torch.float32
        if name == "field":
            # rows of nX = n rounded up to 4, n the particle count of the last kick
            n = self.cap if n is None else int(n)
            nX = (n + 3) // 4 * 4
            return raw.view(dt)[:3 * nX].view(3, nX)[:, :n]
        return raw.view(dt).view(self.shape)

    def profile(self, enable: bool = True):
        N.check(self.lib.sc_profile_enable(self.plan, 1 if enable else 0))

    def launches(self) -> int:
        """Kernels launched by the last kick (host bookkeeping)."""
        return int(self.lib.sc_kick_launches(self.plan))

    def profile_read(self):
        """{stage: ms} of the last kick and the number of kernels it launched (synchronous)."""
        ms = (C.c_float * N.SC_NSTAGES)()
        nl = C.c_int()
        N.check(self.lib.sc_profile_read(self.plan, ms, C.byref(nl)))
        names = [self.lib.sc_profile_stage_name(i).decode() for i in range(N.SC_NSTAGES)]
        return dict(zip(names, [float(v) for v in ms])), nl.value

    def apply_tuning(self, n: int):
        """Launch shapes of the tuning table's entry for this form, mesh and
        particle count (nothing unless the engine is tuned); results do not
        change."""
        if self.tuned and self._tuned_n != n:
            from . import tuning
            for param, value in tuning.lookup(self.precision, self.shape, n).items():
                self.set_param(param, value)
            self._tuned_n = n

    def set_param(self, param: int, value: int):
        """A launch-shape parameter of the plan (N.SC_PARAM_*); results do not change."""
        N.check(self.lib.sc_plan_set_param(self.plan, int(param), int(value)))

    def get_param(self, param: int) -> int:
        v = C.c_int()
        N.check(self.lib.sc_plan_get_param(self.plan, int(param), C.byref(v)))
        return v.value

    def set_wait_limit(self, kernel: int = -1, tries: int = -1):
        """Iteration limit of the bulk-copy waits of one FP32 kernel
        (N.SC_WAIT_FRAME, _EXTENT, _KICK) or of all three (-1) for later
        kicks; tries < 0 restores the default.  A wait that runs out latches
        SC_ERR_TIMEOUT (raised by ``check_status``) instead of spinning on."""
        N.check(self.lib.sc_plan_set_wait_limit(self.plan, int(kernel), int(tries)))

    def check_status(self):
        """Wait for the stream and raise if the last call latched an error."""
        torch = _torch()
        if self.ws is None:
            return
        with torch.cuda.device(self.device):
            N.check(self.lib.sc_read_status(self.plan, _ptr(self.ws), _stream(self.device)))


class SpaceCharge(PhysProc):
    """3D space-charge kick (Ocelot's ``SpaceCharge``, sc.py:76-258).

    Attributes as in the reference: ``step`` (in Navigator unit steps),
    ``nmesh_xyz`` (default [63, 63, 63]), ``low_order_kick`` (stored, unused,
    as in the reference), ``random_mesh``, ``random_seed`` (10), ``debug``,
    ``start_elem``/``end_elem``.  Additions: ``precision`` ("fp64" | "fp32"),
    for the FP32 form ``deposit`` ("fixed": exact 64-bit fixed-point
    accumulation, default; "sorted": radix sort + Kahan segment sums) and
    ``igf`` ("hybrid": FP64 8-corner IGF near the origin, multipole form
    beyond 5 cell widths, default; "exact": FP64 8-corner IGF everywhere),
    ``fields`` ("spectral", default: the forward differences of the
    potential (sc.py:195-200) taken in Fourier space before the inverse
    transforms, so that their FP32 rounding is relative to the field and not
    to the potential, which is hundreds of times larger than the difference
    of neighbouring cells -- ~30x smaller kick errors for ~2% more time on the
    2M / 64^3 beam; "difference": the reference's differences of the FP32
    potential) and ``device``.
    """

    def __init__(self, step=1, **kwargs):
        PhysProc.__init__(self)
        self.step = step
        self.nmesh_xyz = kwargs.get("nmesh_xyz", [63, 63, 63])
        self.low_order_kick = kwargs.get("low_order_kick", True)
        self.start_elem = None
        self.end_elem = None
        self.debug = False
        self.random_mesh = kwargs.get("random_mesh", False)
        self.random_seed = 10
        self.precision = kwargs.get("precision", "fp64")
        self.deposit = kwargs.get("deposit", "fixed")
        self.igf = kwargs.get("igf", "hybrid")
        self.fields = kwargs.get("fields", "spectral")
        plan_mode(self.precision, self.deposit, self.igf, self.fields)  # validates
        self.device = kwargs.get("device", None)
        self._engines = {}

    # ---- plugin hooks -------------------------------------------------
    def prepare(self, lat):
        """sc.py:104-107: check the step and seed numpy's global RNG."""
        self.check_step()
        if self.random_seed is not None:
            np.random.seed(self.random_seed)

    def engine(self, shape=None) -> Engine:
        shape = tuple(int(v) for v in (self.nmesh_xyz if shape is None else shape))
        mode = plan_mode(self.precision, self.deposit, self.igf, self.fields)
        key = (shape, mode, str(self.device))
        eng = self._engines.get(key)
        if eng is None:
            eng = Engine(shape, self.precision, self.device, mode)
            self._engines[key] = eng
        return eng

    def _mesh_draws(self):
        # the two draws of sc.py:174-175 and 184-185, in that order
        if not self.random_mesh:
            return math.nan, math.nan
        scale = np.random.uniform(low=1, high=1.1)
        shift = np.random.uniform(low=-0.5, high=0.5)
        return float(scale), float(shift)

    def apply(self, p_array, zstep):
        """One kick of length ``zstep`` [m] on ``p_array`` in place (sc.py:208-251)."""
        if zstep == 0:
            return
        torch = _torch()
        rp = p_array.rparticles
        if isinstance(rp, torch.Tensor):
            self.apply_device(rp, p_array.q_array, p_array.E, zstep)
            return
        if rp.ndim != 2 or rp.shape[0] != 6:
            raise ValueError(f"rparticles must have shape (6, N), not {rp.shape}")
        n = rp.shape[1]
        if n == 0:
            raise ValueError("zero-size array: the space-charge kick needs at least one particle")
        scale, shift = self._mesh_draws()
        eng = self.engine()
        d_rp, d_q = eng.staging(n)
        src = rp if (rp.dtype == np.float64 and rp.flags.c_contiguous) else np.ascontiguousarray(rp, dtype=np.float64)
        h_rp = torch.from_numpy(src)
        h_q = torch.from_numpy(np.ascontiguousarray(p_array.q_array, dtype=np.float64))
        if h_q.numel() != n:
            raise ValueError(f"q_array has {h_q.numel()} entries for {n} particles")
        with torch.cuda.device(eng.device):
            d_rp.copy_(h_rp, non_blocking=True)
            d_q.copy_(h_q, non_blocking=True)
            eng.kick(d_rp, d_q, n, p_array.E, zstep, scale, shift)
            if src is rp:
                # queued behind the kick; check_status waits once for both.  A
                # kick that stops on an error leaves the device copy as it was
                # copied in, so the caller's values come back unchanged.
                h_rp.copy_(d_rp, non_blocking=True)
                eng.check_status()
            else:
                eng.check_status()
                rp[...] = d_rp.cpu().numpy()

    def apply_device(self, rparticles, q_array, energy_gev, zstep, mesh_draws=None):
        """Kick GPU-resident tensors in place; asynchronous on the current stream.

        Device-side errors are latched; ``check()`` raises them.
        """
        if zstep == 0:
            return
        n = int(rparticles.shape[1])
        if n == 0:
            raise ValueError("zero-size array: the space-charge kick needs at least one particle")
        scale, shift = self._mesh_draws() if mesh_draws is None else mesh_draws
        self.engine().kick(rparticles, q_array, n, energy_gev, zstep, scale, shift)

    def check(self):
        for eng in self._engines.values():
            eng.check_status()

    # ---- the reference's public stage methods, on the GPU ---------------
    def sym_kernel(self, ijk2, hxyz):
        """IGF on the lag octant (sc.py:109-133), FP64, returned as numpy."""
        torch = _torch()
        shape = tuple(int(v) for v in ijk2)
        eng = self.engine(shape)
        eng.ensure(0)
        out = torch.empty(shape, dtype=torch.float64, device=eng.device)
        with torch.cuda.device(eng.device):
            N.check(eng.lib.sc_sym_kernel(eng.plan, _ptr(eng.ws), eng.ws.numel(), float(hxyz[0]), float(hxyz[1]),
                                          float(hxyz[2]), _ptr(out), _stream(eng.device)))
        return out.cpu().numpy()

    def potential(self, q, steps):
        """Potential of a charge grid (sc.py:135-168), returned as numpy."""
        torch = _torch()
        q = np.ascontiguousarray(q, dtype=np.float64)
        eng = self.engine(q.shape)
        eng.ensure(0)
        dq = torch.from_numpy(q).to(eng.device)
        out = torch.empty(q.shape, dtype=torch.float64, device=eng.device)
        with torch.cuda.device(eng.device):
            N.check(eng.lib.sc_potential(eng.plan, _ptr(eng.ws), eng.ws.numel(), _ptr(dq), float(steps[0]),
                                         float(steps[1]), float(steps[2]), _ptr(out), _stream(eng.device)))
            eng.check_status()
        return out.cpu().numpy()

    def el_field(self, X, Q, gamma, nxyz):
        """Rest-frame field at the particles (sc.py:170-205).

        ``X`` [N, 3] is modified in place as the reference modifies it
        (z scaled by gamma); returns Exyz [N, 3].
        """
        torch = _torch()
        scale, shift = self._mesh_draws()
        eng = self.engine(nxyz)
        n = X.shape[0]
        eng.ensure(n)
        dX = torch.from_numpy(np.ascontiguousarray(X, dtype=np.float64)).to(eng.device)
        dQ = torch.from_numpy(np.ascontiguousarray(Q, dtype=np.float64)).to(eng.device)
        out = torch.empty((n, 3), dtype=torch.float64, device=eng.device)
        with torch.cuda.device(eng.device):
            N.check(eng.lib.sc_el_field(eng.plan, _ptr(eng.ws), eng.ws.numel(), _ptr(dX), _ptr(dQ), n, float(gamma),
                                        scale, shift, _ptr(out), _stream(eng.device)))
            eng.check_status()
        X[...] = dX.cpu().numpy()
        return out.cpu().numpy()

    def __repr__(self) -> str:
        cname = type(self).__name__
        step = self.step
        nmesh_xyz = self.nmesh_xyz
        random_mesh = self.random_mesh
        return f"<{cname}: {step=}, {nmesh_xyz=}, {random_mesh=}>"
