"""Device-resident tracking: first-order transport plus space-charge kicks,
with the particles kept on the GPU from the first step to the last.

The reference tracks with ``track(lat, p_array, navi)``
(ocelot/cpbd/track.py:431-505): for every step its Navigator builds the
element slices up to the next kick (navi.py:343-434), each slice map is
applied to ``rparticles`` (TransferMap.mul_p_array,
transformations/transfer_map.py:40-50) and then the kick runs
(SpaceCharge.apply).  Here the same schedule is computed once on the host,
the slice maps of each step are composed into one 6x6 map, the maps are
stored in a device table, and every step is two calls on the job's stream:
``sc_tmap_apply_indexed`` (map ``*counter``, then ``*counter += 1``) and
``sc_kick``.  Because the map index lives on the device, the launches of one
step are recorded once as a CUDA graph and replayed for every step of equal
kick length (all but the last, truncated one, in a uniform lattice).

Scope: drifts, quadrupoles (with tilt and offsets), markers and monitors --
the elements whose first-order map is ``uni_matrix`` without bending
(ocelot/cpbd/r_matrix.py:41-91); one SpaceCharge process attached from the
first to the last element, the configuration of a space-charge transport
line.  With ``order=2`` the transport is the reference's SecondTM instead
(second_order.py): the slices of a step are not composed but applied one
after the other in one pass (``sc_tmap2_apply_step``).
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _native as N
from .globals import m_e_GeV


# ---------------------------------------------------------------------------
# Elements
# ---------------------------------------------------------------------------
class Element:
    """Drift-like element with a first-order map (length l [m])."""

    def __init__(self, l=0.0, eid=None):
        self.l = float(l)
        self.k1 = 0.0
        self.tilt = 0.0
        self.angle = 0.0
        self.dx = 0.0
        self.dy = 0.0
        self.id = eid


class Drift(Element):
    pass


class Marker(Element):
    def __init__(self, eid=None):
        super().__init__(0.0, eid)


class Quadrupole(Element):
    def __init__(self, l=0.0, k1=0.0, tilt=0.0, eid=None):
        super().__init__(l, eid)
        self.k1 = float(k1)
        self.tilt = float(tilt)


_SUPPORTED = ("Drift", "Marker", "Monitor", "Quadrupole", "Element")


def _element_params(e):
    """(length, k1, tilt, dx, dy) of a drift/quadrupole/marker, from this
    module's classes or any object with the reference's element attributes."""
    name = type(e).__name__
    if name not in _SUPPORTED:
        raise NotImplementedError(f"{name}: device tracking supports drifts, quadrupoles, markers and monitors")
    angle = float(getattr(e, "angle", 0.0) or 0.0)
    if angle != 0.0:
        raise NotImplementedError(f"{name} with angle {angle}: bends are not supported by device tracking")
    return (float(e.l), float(getattr(e, "k1", 0.0) or 0.0), float(getattr(e, "tilt", 0.0) or 0.0),
            float(getattr(e, "dx", 0.0) or 0.0), float(getattr(e, "dy", 0.0) or 0.0))


# ---------------------------------------------------------------------------
# First-order maps
# ---------------------------------------------------------------------------
def first_order_matrix(length: float, k1: float, energy: float) -> np.ndarray:
    """6x6 first-order matrix of an unbent drift (k1 = 0) or quadrupole of
    ``length`` [m] at ``energy`` [GeV]: the reference's uni_matrix
    (ocelot/cpbd/r_matrix.py:41-91) at hx = 0, written with real
    cos/sin (k1 > 0) and cosh/sinh (k1 < 0) instead of complex roots.  The
    only longitudinal term is R56 = -L / (beta^2 gamma^2)."""
    z = float(length)
    gamma = energy / m_e_GeV
    ig2 = 1.0 / (gamma * gamma) if gamma != 0 else 0.0
    beta2 = 1.0 - ig2

    def cs(k2):
        if k2 > 0:
            w = math.sqrt(k2)
            return math.cos(w * z), math.sin(w * z) / w
        if k2 < 0:
            w = math.sqrt(-k2)
            return math.cosh(w * z), math.sinh(w * z) / w
        return 1.0, z

    cx, sx = cs(k1)
    cy, sy = cs(-k1)
    R = np.eye(6)
    R[0, 0], R[0, 1], R[1, 0], R[1, 1] = cx, sx, -k1 * sx, cx
    R[2, 2], R[2, 3], R[3, 2], R[3, 3] = cy, sy, k1 * sy, cy
    R[4, 5] = -z / beta2 * ig2
    return R


def _rotation(angle: float) -> np.ndarray:
    c, s = math.cos(angle), math.sin(angle)
    m = np.eye(6)
    m[0, 0] = m[1, 1] = m[2, 2] = m[3, 3] = c
    m[0, 2] = m[1, 3] = s
    m[2, 0] = m[3, 1] = -s
    return m


def element_map(e, length: float, energy: float):
    """(R, B) of a ``length`` section of element ``e``: tilt applied as
    rot(-tilt).R.rot(tilt) (tm_params/first_order_params.py:26-28), offsets as
    B = (I - R).(dx, 0, dy, 0, 0, 0) (elements/element.py:80-81)."""
    _, k1, tilt, dx, dy = _element_params(e)
    R0 = first_order_matrix(length, k1, energy)
    B = (np.eye(6) - R0) @ np.array([dx, 0.0, dy, 0.0, 0.0, 0.0])
    R = _rotation(-tilt) @ R0 @ _rotation(tilt) if tilt != 0.0 else R0
    return R, B


# ---------------------------------------------------------------------------
# The Navigator's kick schedule
# ---------------------------------------------------------------------------
def _section_length(total: float, start: float, want: float) -> float:
    # the length OpticElement.get_section_tms builds a slice map for
    # (elements/optic_element.py:376-403)
    if start < 1e-10 and np.isclose(want, total):
        return total
    if start + want > total or np.isclose(start + want, total):
        return total - start
    return want


def kick_schedule(lengths, unit_step: float, step: int = 1):
    """Kicks of one SpaceCharge process attached from the first to the last
    element: [(slices, zstep, z0)], slices = [(element index, length)] to
    transport before the kick of length ``zstep`` at position ``z0``.

    The positions are accumulated with the floating-point operations of the
    reference's Navigator (ocelot/cpbd/navi.py:219-237, 343-371, 406-434;
    lattice length as MagneticLattice.totalLen, magnetic_lattice.py:226-227,
    stop position as add_physics_proc, navi.py:76-77), so the kick lengths
    and slice boundaries are the reference's to the last bit.
    """
    lengths = [float(v) for v in lengths]
    if not lengths:
        raise ValueError("empty lattice")
    nel = len(lengths)
    total = 0.0
    for v in lengths:
        total += v
    stop = float(np.sum(np.array(lengths[:nel - 1]))) if nel > 1 else 0.0
    nominal = float(step) * float(unit_step)
    if not nominal > 0:
        raise ValueError("unit_step * step must be positive")
    z, elem, before = 0.0, 0, 0.0
    out = []
    while abs(z - total) > 1e-10:
        dz = nominal
        if z + dz > stop:
            dz = stop - z
        if not dz > 0:
            raise ValueError("the space-charge process range ends before the lattice does")
        zstep = (nominal - nominal) + dz
        if z + dz > total:
            dz = total - z
        # walk the elements up to z + dz
        i, end, left, slices = elem, z + dz, dz, []
        edge = before + lengths[i]
        while end + 1e-10 > edge:
            dl = edge - z
            slices.append((i, _section_length(lengths[i], z + lengths[i] - edge, dl)))
            z = edge
            left -= dl
            if i >= nel - 1:
                break
            i += 1
            edge += lengths[i]
        if abs(left) > 1e-10:
            slices.append((i, _section_length(lengths[i], z + lengths[i] - edge, left)))
        z += left
        before, elem = edge - lengths[i], i
        out.append((slices, zstep, z))
        if len(out) > 10_000_000:
            raise RuntimeError("kick schedule does not terminate")
    return out


def step_maps(elements, energy: float, unit_step: float, step: int = 1):
    """Composed map (R, B) and kick (zstep, z0) of every step."""
    lengths = [_element_params(e)[0] for e in elements]
    steps = []
    for slices, zstep, z0 in kick_schedule(lengths, unit_step, step):
        R, B = np.eye(6), np.zeros(6)
        for i, dl in slices:
            if dl == 0.0:
                continue
            Ri, Bi = element_map(elements[i], dl, energy)
            R, B = Ri @ R, Ri @ B + Bi
        steps.append((R, B, zstep, z0))
    return steps


def step_maps2(elements, energy: float, unit_step: float, step: int = 1):
    """Second-order maps of every step: (packed slice maps [m, MAP2_DOUBLES],
    zstep, z0), the slices in the order the reference applies them."""
    from .second_order import MAP2_DOUBLES, element_map2, pack_map
    lengths = [_element_params(e)[0] for e in elements]
    steps = []
    for slices, zstep, z0 in kick_schedule(lengths, unit_step, step):
        maps = [pack_map(*element_map2(elements[i], dl, energy)) for i, dl in slices if dl != 0.0]
        steps.append((np.array(maps).reshape(-1, MAP2_DOUBLES), zstep, z0))
    return steps


def lattice_order(lat) -> int:
    """2 when the reference lattice tracks with SecondTM (its ``method``
    dict), else 1."""
    method = getattr(lat, "method", None)
    glob = method.get("global") if isinstance(method, dict) else None
    return 2 if glob is not None and getattr(glob, "__name__", "") == "SecondTM" else 1


# ---------------------------------------------------------------------------
# The device loop
# ---------------------------------------------------------------------------
def _lattice_sequence(lat):
    return list(lat.sequence) if hasattr(lat, "sequence") else list(lat)


class DeviceTrack:
    """One tracking job resident on the GPU: its particles, its map table,
    the kick's plan and workspace (Green's table cache included) and its own
    stream.  ``step()`` enqueues the next step; ``run()`` all of them.

    ``elements``: drifts/quadrupoles/markers (a lattice object with
    ``.sequence`` or a list); ``sc``: the SpaceCharge process (its precision,
    mesh and deposit/IGF options are used; random_mesh is not supported,
    its draws would have to be taken per step on the host); ``unit_step``:
    the Navigator's unit step; ``p_array``: host ParticleArray or
    DeviceParticleArray (the particles are copied once to the device).
    """

    def __init__(self, elements, sc, unit_step: float, p_array, graph: bool = True, stream=None, order: int = 1):
        import torch
        from .beam import DeviceParticleArray
        from .sc import Engine, plan_mode
        if sc.random_mesh:
            raise NotImplementedError("random_mesh draws host random numbers per kick: use track() on the host")
        seq = _lattice_sequence(elements)
        self.dev = torch.device(sc.device) if sc.device is not None else torch.device(
            "cuda", torch.cuda.current_device())
        if isinstance(p_array, DeviceParticleArray):
            self.beam = p_array
        else:
            self.beam = DeviceParticleArray.from_host(p_array, self.dev)
        self.n = int(self.beam.rparticles.shape[1])
        if self.n == 0:
            raise ValueError("zero-size array: the space-charge kick needs at least one particle")
        self.E = float(self.beam.E)
        if order not in (1, 2):
            raise ValueError("order must be 1 (TransferMap) or 2 (SecondTM)")
        self.order = order
        if order == 1:
            self.steps = step_maps(seq, self.E, unit_step, int(sc.step))
            table = np.zeros((len(self.steps), 42))
            for k, (R, B, _, _) in enumerate(self.steps):
                table[k, :36] = R.reshape(-1)
                table[k, 36:] = B
        else:
            # the slice maps of all steps, and where each step's maps begin
            steps2 = step_maps2(seq, self.E, unit_step, int(sc.step))
            self.steps = [(None, None, zstep, z0) for _, zstep, z0 in steps2]
            table = np.concatenate([m for m, _, _ in steps2]) if steps2 else np.zeros((0, 1))
            first = np.cumsum([0] + [m.shape[0] for m, _, _ in steps2]).astype(np.int32)
            self.first = torch.from_numpy(first).to(self.dev)
        self.table = torch.from_numpy(np.ascontiguousarray(table)).to(self.dev)
        self.counter = torch.zeros(1, dtype=torch.int32, device=self.dev)
        self.engine = Engine(tuple(int(v) for v in sc.nmesh_xyz), sc.precision, self.dev,
                             plan_mode(sc.precision, sc.deposit, sc.igf))
        self.engine.ensure(self.n)
        self.stream = stream if stream is not None else torch.cuda.Stream(self.dev)
        self.next = 0
        self.use_graph = bool(graph)
        self._graphs = {}
        self.done = torch.cuda.Event()
        with torch.cuda.device(self.dev):
            self.stream.wait_stream(torch.cuda.current_stream(self.dev))

    @property
    def nsteps(self) -> int:
        return len(self.steps)

    @property
    def finished(self) -> bool:
        return self.next >= len(self.steps)

    def _launch(self, zstep: float):
        import torch
        rp, q = self.beam.rparticles, self.beam.q_array
        lib = self.engine.lib
        s = C.c_void_p(torch.cuda.current_stream(self.dev).cuda_stream)
        if self.order == 1:
            N.check(lib.sc_tmap_apply_indexed(C.c_void_p(self.table.data_ptr()), C.c_void_p(self.counter.data_ptr()),
                                              len(self.steps), C.c_void_p(rp.data_ptr()), rp.stride(0), self.n, s))
        else:
            N.check(lib.sc_tmap2_apply_step(C.c_void_p(self.table.data_ptr()), C.c_void_p(self.first.data_ptr()),
                                            C.c_void_p(self.counter.data_ptr()), len(self.steps),
                                            C.c_void_p(rp.data_ptr()), rp.stride(0), self.n, s))
        self.engine.kick(rp, q, self.n, self.E, zstep)

    def _graph(self, zstep: float):
        import torch
        g = self._graphs.get(zstep)
        if g is None:
            g = torch.cuda.CUDAGraph()
            with torch.cuda.device(self.dev):
                self.stream.synchronize()
                # recording does not execute: counter and particles are untouched
                with torch.cuda.graph(g, stream=self.stream):
                    self._launch(zstep)
            self._graphs[zstep] = g
        return g

    def step(self, count: int = 1) -> int:
        """Enqueue up to ``count`` steps on the job's stream (asynchronous);
        returns how many were enqueued."""
        import torch
        k = 0
        with torch.cuda.device(self.dev), torch.cuda.stream(self.stream):
            while k < count and self.next < len(self.steps):
                zstep = self.steps[self.next][2]
                if self.use_graph:
                    self._graph(zstep).replay()
                else:
                    self._launch(zstep)
                self.next += 1
                k += 1
            if self.next >= len(self.steps) and k:
                self.done.record(self.stream)
        return k

    def run(self):
        self.step(len(self.steps))
        return self

    def synchronize(self):
        """Wait for the job and raise if any of its kicks latched an error."""
        import torch
        self.stream.synchronize()
        with torch.cuda.device(self.dev), torch.cuda.stream(self.stream):
            self.engine.check_status()
            first = int(self.engine.region("first_error").item())
        if first:
            raise ValueError(f"[sc error {first}] {N.ERROR_TEXT.get(first, 'device error')} (in an earlier step)")

    def result(self, p_array=None):
        self.synchronize()
        self.beam.s = self.steps[-1][3] if self.steps else self.beam.s
        return self.beam.to_host(p_array)


def track(lattice, p_array, navi=None, sc=None, unit_step=None, graph: bool = True, order=None):
    """Device counterpart of the reference's ``track(lat, p_array, navi)``
    for a space-charge transport line: the particles go to the GPU once, all
    steps run there, and ``p_array`` is updated in place at the end.

    Either pass a Navigator-like ``navi`` (``unit_step`` and one SpaceCharge
    process in ``navi.process_table.proc_list``) or ``sc`` and ``unit_step``.
    ``order``: 1 (first-order maps, TransferMap) or 2 (SecondTM); by default
    the lattice's own ``method`` decides.
    Returns (tws, p_array) like the reference, with an empty twiss list.
    """
    if navi is not None:
        procs = []
        for table in ("process_table", "ref_process_table"):
            procs += [p for p in (getattr(getattr(navi, table, None), "proc_list", None) or []) if p not in procs]
        if sc is None:
            from .sc import SpaceCharge
            found = [p for p in procs if isinstance(p, SpaceCharge)]
            if len(found) != 1:
                raise NotImplementedError("device tracking takes exactly one ocelot_gb300 SpaceCharge process")
            sc = found[0]
            seq = _lattice_sequence(lattice)
            i0, i1 = getattr(sc, "indx0", None), getattr(sc, "indx1", None)
            if (i0 is not None and i0 != 0) or (i1 is not None and i1 != len(seq) - 1):
                raise NotImplementedError("device tracking needs the SpaceCharge process on the whole lattice")
        unit_step = navi.unit_step if unit_step is None else unit_step
    if sc is None or unit_step is None:
        raise ValueError("pass navi, or sc and unit_step")
    order = lattice_order(lattice) if order is None else int(order)
    job = DeviceTrack(lattice, sc, unit_step, p_array, graph=graph, order=order).run()
    job.result(p_array)
    return [], p_array
