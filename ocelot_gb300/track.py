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
(ocelot/cpbd/r_matrix.py:41-91) -- and standing-wave RF cavities (CavityTM,
``cavity.py``); any number of SpaceCharge processes, each over its element
range with its own step count.  With one process over a line without
cavities and first-order maps, each step's slice maps are composed into one.
With ``order=2`` the transport is the reference's SecondTM instead
(second_order.py), and in a line with cavities or several processes the
slices of a step are not composed but applied one after the other in one
pass (``sc_slices_apply_step``), the beam energy carried through the
cavities.  ``track()`` also returns the twiss list (beam moments taken on
the device after every step, ``envelope.py``).
"""
from __future__ import annotations

import ctypes as C
import math
from typing import NamedTuple

import numpy as np

from . import _native as N
from .cavity import Cavity  # noqa: F401  (the line elements are importable from here)
from .envelope import Twiss  # noqa: F401
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
        raise NotImplementedError(f"{name}: device tracking supports drifts, quadrupoles, markers, monitors and "
                                  "cavities")
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
    # MagneticLattice.totalLen is the built-in sum() of the lengths (compensated
    # summation on Python 3.12+), not a running total
    total = sum(lengths)
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


def navigator_steps(lengths, procs, unit_step: float):
    """The steps of a Navigator with several processes, each attached over
    elements [indx0, indx1) with its own step count: a list of
    (sections, kicks, z0, dz), sections = [(element index, start in the
    element, length)] transported in the step, kicks = [(process index, zstep)]
    applied after it, in the reference's order, z0 the position after the step
    and dz the step length get_next_step yields (track() adds it to the twiss
    position).
    ``procs`` = [(indx0, indx1, step)] in the order the processes were added.

    Restates Navigator.get_next_step / get_next / check_overjump /
    check_proc_bounds / get_map (ocelot/cpbd/navi.py:343-352, 354-390,
    219-266, 281-287, 406-434) with the positions of add_physics_proc
    (navi.py:58-64) and MagneticLattice.totalLen; processes on a single
    element (the Navigator's kick processes) are not supported.
    """
    lengths = [float(v) for v in lengths]
    nel = len(lengths)
    if not nel:
        raise ValueError("empty lattice")
    procs = [(int(a), int(b), int(st)) for a, b, st in procs]
    for a, b, st in procs:
        if not (0 <= a < nel and 0 <= b < nel and a <= b):
            raise ValueError(f"process range [{a}, {b}) is not inside the lattice")
        if a == b or (a + 1 == b and lengths[a] == 0):
            raise NotImplementedError("a process on a single element (a kick process) is not supported")
        if st < 1:
            raise ValueError("process step must be >= 1")
    total = sum(lengths)      # MagneticLattice.totalLen (magnetic_lattice.py:225-227)
    s_start = [np.sum(np.array(lengths[:a])) for a, _, _ in procs]
    s_stop = [np.sum(np.array(lengths[:b])) for _, b, _ in procs]
    counters = [st for _, _, st in procs]
    z0, n_elem, sum_lengths = 0.0, 0, 0.0
    out = []
    while np.abs(z0 - total) > 1e-10:
        active = [j for j, (a, b, _) in enumerate(procs) if a <= n_elem < b]
        if active:
            cmin = min(counters[j] for j in active)
            chosen = [j for j in active if counters[j] == cmin]
            phys = np.array([procs[j][2] for j in chosen]) * unit_step
            for j in active:
                counters[j] -= cmin
                if counters[j] == 0:
                    counters[j] = procs[j][2]
            dz = np.min(phys)
        else:
            chosen = []
            dz = (np.sum(np.array(lengths[:n_elem + 1])) if nel >= n_elem + 1 else total) - z0
            phys = np.array([])
        phys_red = phys - dz
        if chosen:
            l_stop = np.sum(np.array(lengths[:min(procs[j][1] for j in chosen)]))
            if z0 + dz > l_stop:
                dz = l_stop - z0
            starts = sorted(s_start[j] for j in range(len(procs)) if j not in chosen and z0 < s_start[j] < z0 + dz)
            if starts:
                dz = starts[0] - z0
        phys = phys_red + dz
        for j in active:
            if dz + z0 >= s_stop[j] and j not in chosen:
                chosen.append(j)
                phys = np.append(phys, dz)
        if z0 + dz > total:
            dz = total - z0
        step_dz = float(dz)
        # Navigator.get_map
        sections, i = [], n_elem
        z1 = z0 + dz
        L = sum_lengths + lengths[i]
        while z1 + 1e-10 > L:
            dl = L - z0
            sections.append((i, z0 + lengths[i] - L, dl))
            z0 = L
            dz -= dl
            if i >= nel - 1:
                break
            i += 1
            L += lengths[i]
        if abs(dz) > 1e-10:
            sections.append((i, z0 + lengths[i] - L, dz))
        z0 += dz
        sum_lengths = L - lengths[i]
        n_elem = i
        out.append((sections, [(j, float(phys[q])) for q, j in enumerate(chosen)], float(z0), step_dz))
        if len(out) > 10_000_000:
            raise RuntimeError("the Navigator's schedule does not terminate")
    return out


def _line_lengths(seq):
    from .cavity import is_cavity
    return [float(e.l) if is_cavity(e) else _element_params(e)[0] for e in seq]


class StepSlices(NamedTuple):
    table: np.ndarray      # [m, MAP2_DOUBLES] records
    kinds: np.ndarray      # [m] SLICE_MAP | SLICE_CAVITY
    kicks: list            # [(process, energy, zstep)]
    z0: float              # Navigator position after the step
    E: float               # beam energy after the step's maps
    dz: float              # step length


def step_slices(elements, energy: float, steps, order: int = 2, s: float = 0.0):
    """Device records of the maps of every step of ``steps`` (from
    navigator_steps), with the reference energy carried through the cavities
    as Transformation.apply does (p_array.E += delta_e after every map):
    ([StepSlices], final energy, final position).  The position is accumulated as
    Transformation.apply moves p_array.s: by each map's length, starting
    from ``s``.  Drift/quadrupole slices are SecondTM maps (order 2) or
    first-order maps with T = 0 (order 1); cavity sections are the coupler
    kicks (left out when they are the identity, which the reference applies
    exactly) and the cavity slice records."""
    from . import cavity as CV
    from .second_order import element_map2, pack_map
    zero_t = np.zeros((6, 6, 6))
    E = energy
    out = []
    for sections, kicks, z0, dz in steps:
        recs, kinds = [], []
        for i, start_l, dl in sections:
            e = elements[i]
            if CV.is_cavity(e):
                r, k, E = CV.section_records(e, start_l, dl, E)
                recs += list(r)
                kinds += k
                for kind, d in CV.section_tms(e, start_l, dl, True):
                    s += (d if d is not None else e.l) if kind == "main" else 0.0
                continue
            length = _section_length(e.l, start_l, dl)
            s += length
            if length == 0.0:
                continue
            if order == 2:
                recs.append(pack_map(*element_map2(e, length, E)))
            else:
                R, B = element_map(e, length, E)
                recs.append(pack_map(R, zero_t, B))
            kinds.append(CV.map_kind(recs[-1]))
        table = np.array(recs).reshape(-1, CV.MAP2_DOUBLES)
        out.append(StepSlices(table, np.array(kinds, dtype=np.int32), [(j, E, zstep) for j, zstep in kicks], z0, E,
                              dz))
    return out, E, s


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
    the kicks' plans and workspaces (Green's table caches included) and its
    own stream.  ``step()`` enqueues the next step; ``run()`` all of them.

    ``elements``: drifts/quadrupoles/markers/cavities (a lattice object with
    ``.sequence`` or a list); ``sc``: the SpaceCharge process attached from
    the first to the last element, or ``processes`` = [(SpaceCharge, indx0,
    indx1)], each attached over elements [indx0, indx1) as
    Navigator.add_physics_proc does, in the order they were added (each
    process's precision, mesh, deposit/IGF options and random_mesh are used;
    the random mesh draws are taken when the job is built, in kick order);
    ``unit_step``: the Navigator's unit step; ``p_array``: host ParticleArray
    or DeviceParticleArray (the particles are copied once to the device).

    A line of drifts and quadrupoles with one process over all of it and
    first-order maps composes each step's slices into one map
    (``sc_tmap_apply_indexed``).  Otherwise -- second-order maps, cavities,
    several processes -- each step's slices are applied one after the other
    in one pass (``sc_slices_apply_step``), the reference energy is carried
    through the cavities on the host, and each kick gets the energy of its
    step.  Steps whose kicks (energy, length, plan) repeat are recorded once
    as a CUDA graph and replayed.

    ``twiss``: take the beam moments on the device before the first step and
    after every step (``sc_moments``, get_envelope's statistics; ``bounds`` =
    [lo, hi] selects the particles within lo..hi standard deviations of tau
    around its mean); ``twiss_list()`` returns them as Twiss objects.
    """

    def __init__(self, elements, sc, unit_step: float, p_array, graph: bool = True, stream=None, order: int = 1,
                 processes=None, twiss: bool = False, bounds=None):
        import torch
        from .beam import DeviceParticleArray
        from .cavity import is_cavity
        seq = _lattice_sequence(elements)
        if processes is None:
            if sc is None:
                raise ValueError("pass sc or processes")
            processes = [(sc, 0, len(seq) - 1)]
            whole = True
        else:
            processes = [(p, int(a), int(b)) for p, a, b in processes]
            if not processes:
                raise ValueError("processes is empty: device tracking needs at least one SpaceCharge process")
            whole = len(processes) == 1 and processes[0][1] == 0 and processes[0][2] == len(seq) - 1
        p0 = processes[0][0]
        self.dev = torch.device(p0.device) if p0.device is not None else torch.device(
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
        lengths = _line_lengths(seq)
        self.composed = order == 1 and whole and not any(is_cavity(e) for e in seq)
        self.engines, eng_of = [], []
        from .sc import Engine, plan_mode
        keys = {}
        for p, _, _ in processes:
            key = (tuple(int(v) for v in p.nmesh_xyz), p.precision,
                   plan_mode(p.precision, p.deposit, p.igf, getattr(p, "fields", "spectral")))
            if key not in keys:
                keys[key] = len(self.engines)
                self.engines.append(Engine(key[0], key[1], self.dev, key[2]))
            eng_of.append(keys[key])
        self.engine = self.engines[0]
        for eng in self.engines:
            eng.ensure(self.n)
        if self.composed:
            self.steps = []
            maps = step_maps(seq, self.E, unit_step, int(processes[0][0].step))
            table = np.zeros((len(maps), 42))
            for k, (R, B, zstep, z0) in enumerate(maps):
                table[k, :36] = R.reshape(-1)
                table[k, 36:] = B
                self.steps.append((((0, self.E, zstep) + self._draws(processes[0][0], zstep),), z0))
            self.E_end = self.E
            self.s_end = float(self.beam.s)
            for slices, _, _ in kick_schedule(lengths, unit_step, int(processes[0][0].step)):
                for _, dl in slices:
                    self.s_end += dl
            self._step_E = [self.E] * len(self.steps)
            # (a two-element line whose first element has no length makes the process a kick process for the
            # reference's Navigator, applied once: not supported, navigator_steps raises)
            self._step_dz = [st[3] for st in navigator_steps(
                lengths, [(0, len(seq) - 1, int(processes[0][0].step))], unit_step)]
        else:
            sched = navigator_steps(lengths, [(a, b, p.step) for p, a, b in processes], unit_step)
            slices, self.E_end, self.s_end = step_slices(seq, self.E, sched, order, float(self.beam.s))
            self.steps = [(tuple((eng_of[j], float(E), float(zstep)) + self._draws(processes[j][0], zstep)
                                 for j, E, zstep in st.kicks), st.z0) for st in slices]
            self._step_E = [float(st.E) for st in slices]
            self._step_dz = [st.dz for st in slices]
            table = np.concatenate([st.table for st in slices]) if slices else np.zeros((0, 1))
            if table.shape[0] == 0:
                table = np.zeros((1, N.SC_MAP2_DOUBLES))
            kinds = np.concatenate([st.kinds for st in slices]) if slices else np.zeros(0, np.int32)
            first = np.cumsum([0] + [st.table.shape[0] for st in slices]).astype(np.int32)
            self.first = torch.from_numpy(first).to(self.dev)
            self.kinds = torch.from_numpy(np.ascontiguousarray(np.append(kinds, 0).astype(np.int32))).to(self.dev)
        self.table = torch.from_numpy(np.ascontiguousarray(table)).to(self.dev)
        self.counter = torch.zeros(1, dtype=torch.int32, device=self.dev)
        self.twiss = bool(twiss)
        self.bounds = None if bounds is None else (float(bounds[0]), float(bounds[1]))
        if self.twiss:
            from .envelope import MOMENTS
            q_host = p_array.q_array if not isinstance(p_array, DeviceParticleArray) else \
                self.beam.q_array.cpu().numpy()
            self.q_total = float(np.sum(np.asarray(q_host)))
            self.moments = torch.zeros((len(self.steps) + 1, MOMENTS), dtype=torch.float64, device=self.dev)
            self._mom_scratch = torch.zeros(int(self.engine.lib.sc_moments_scratch_bytes()), dtype=torch.uint8,
                                            device=self.dev)
        self.stream = stream if stream is not None else torch.cuda.Stream(self.dev)
        self.next = 0
        self.use_graph = bool(graph)
        self._graphs = {}
        # a graph pays when its step repeats (the composed line: every step)
        self._repeats = {}
        for key, _ in self.steps:
            self._repeats[key] = self._repeats.get(key, 0) + 1
        self.done = torch.cuda.Event()
        with torch.cuda.device(self.dev):
            self.stream.wait_stream(torch.cuda.current_stream(self.dev))
            if self.twiss:
                with torch.cuda.stream(self.stream):
                    self._moments(None)      # slot 0: the beam before the first step

    @staticmethod
    def _draws(p, zstep):
        """A random_mesh process's two draws for one kick (sc.py:174-175,
        184-185), taken from numpy's global generator in kick order when the
        job is built -- the order the reference's track() takes them in
        (SpaceCharge.apply returns before drawing when zstep is 0)."""
        if not p.random_mesh or zstep == 0:
            return (None, None)
        scale, shift = p._mesh_draws()
        return (float(scale), float(shift))

    @property
    def nsteps(self) -> int:
        return len(self.steps)

    @property
    def finished(self) -> bool:
        return self.next >= len(self.steps)

    def _launch(self, kicks):
        import torch
        rp, q = self.beam.rparticles, self.beam.q_array
        lib = self.engine.lib
        s = C.c_void_p(torch.cuda.current_stream(self.dev).cuda_stream)
        if self.composed:
            N.check(lib.sc_tmap_apply_indexed(C.c_void_p(self.table.data_ptr()), C.c_void_p(self.counter.data_ptr()),
                                              len(self.steps), C.c_void_p(rp.data_ptr()), rp.stride(0), self.n, s))
        else:
            N.check(lib.sc_slices_apply_step(C.c_void_p(self.table.data_ptr()), C.c_void_p(self.kinds.data_ptr()),
                                             C.c_void_p(self.first.data_ptr()), C.c_void_p(self.counter.data_ptr()),
                                             len(self.steps), C.c_void_p(rp.data_ptr()), rp.stride(0), self.n, s))
        for eng, E, zstep, scale, shift in kicks:
            self.engines[eng].kick(rp, q, self.n, E, zstep, math.nan if scale is None else scale,
                                   math.nan if shift is None else shift)
        if self.twiss:
            self._moments(self.counter)      # slot *counter = step + 1 (advanced by the transport)

    def _moments(self, counter):
        import torch
        rp = self.beam.rparticles
        s = C.c_void_p(torch.cuda.current_stream(self.dev).cuda_stream)
        lo, hi = self.bounds if self.bounds is not None else (0.0, 0.0)
        N.check(self.engine.lib.sc_moments(C.c_void_p(rp.data_ptr()), rp.stride(0), self.n,
                                           None if counter is None else C.c_void_p(counter.data_ptr()),
                                           int(self.moments.shape[0]), 1 if self.bounds is not None else 0, lo, hi,
                                           C.c_void_p(self.moments.data_ptr()), C.c_void_p(self._mom_scratch.data_ptr()),
                                           s))

    def twiss_list(self):
        """Twiss of the beam before the first step and after every step, as
        the reference's track() returns them (s = the sum of the step lengths
        so far, E = the beam energy after the step).  Waits for the job."""
        from .envelope import twiss_from_moments
        if not self.twiss:
            raise RuntimeError("the job was created with twiss=False")
        if not self.finished:
            raise RuntimeError("the job has steps left to run")
        self.synchronize()
        m = self.moments.cpu().numpy()
        out = [twiss_from_moments(m[0], self.E, self.q_total, 0.0)]
        L = 0.
        for k in range(len(self.steps)):
            L += self._step_dz[k]
            out.append(twiss_from_moments(m[k + 1], self._step_E[k], self.q_total, 0.0 + L))
        return out

    def _graph(self, kicks):
        import torch
        g = self._graphs.get(kicks)
        if g is None:
            g = torch.cuda.CUDAGraph()
            with torch.cuda.device(self.dev):
                self.stream.synchronize()
                # recording does not execute: counter and particles are untouched
                with torch.cuda.graph(g, stream=self.stream):
                    self._launch(kicks)
            self._graphs[kicks] = g
        return g

    def step(self, count: int = 1) -> int:
        """Enqueue up to ``count`` steps on the job's stream (asynchronous);
        returns how many were enqueued."""
        import torch
        k = 0
        with torch.cuda.device(self.dev), torch.cuda.stream(self.stream):
            while k < count and self.next < len(self.steps):
                kicks = self.steps[self.next][0]
                if self.use_graph and self._repeats[kicks] > 1:
                    self._graph(kicks).replay()
                else:
                    self._launch(kicks)
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
            for eng in self.engines:
                eng.check_status()
                first = int(eng.region("first_error").item())
                if first:
                    raise ValueError(f"[sc error {first}] {N.ERROR_TEXT.get(first, 'device error')} "
                                     "(in an earlier step)")

    def result(self, p_array=None):
        self.synchronize()
        self.beam.s = self.s_end
        self.beam.E = self.E_end
        return self.beam.to_host(p_array)


def _navigator_processes(navi, lattice):
    """[(process, indx0, indx1)] of a Navigator-like object, in the order the
    processes were added (its process table; a process without the indices
    add_physics_proc sets spans the lattice)."""
    from .sc import SpaceCharge
    procs = []
    for table in ("process_table", "ref_process_table"):
        for p in (getattr(getattr(navi, table, None), "proc_list", None) or []):
            if not any(p is q for q in procs):
                procs.append(p)
    if not procs:
        raise NotImplementedError("device tracking needs at least one ocelot_gb300 SpaceCharge process")
    seq = _lattice_sequence(lattice)
    out = []
    for p in procs:
        if not isinstance(p, SpaceCharge):
            raise NotImplementedError(f"{type(p).__name__}: device tracking runs ocelot_gb300 SpaceCharge processes only")
        i0, i1 = getattr(p, "indx0", None), getattr(p, "indx1", None)
        out.append((p, 0 if i0 is None else int(i0), len(seq) - 1 if i1 is None else int(i1)))
    return out


def track(lattice, p_array, navi=None, sc=None, unit_step=None, graph: bool = True, order=None,
          calc_tws: bool = True, bounds=None, slice=None):
    """Device counterpart of the reference's ``track(lat, p_array, navi)``
    for a space-charge transport line: the particles go to the GPU once, all
    steps run there, and ``p_array`` is updated in place at the end (its
    energy and position included).

    Either pass a Navigator-like ``navi`` (``unit_step`` and its SpaceCharge
    processes in ``navi.process_table.proc_list``, with the element ranges
    add_physics_proc gave them) or ``sc`` and ``unit_step`` (one process over
    the whole lattice).  ``order``: 1 (first-order maps, TransferMap) or 2
    (SecondTM); by default the lattice's own ``method`` decides.  Cavities are
    tracked with their own map (CavityTM) in either case, as in the reference.
    ``calc_tws``, ``bounds``: as the reference's track() -- the beam's Twiss
    before the first step and after each step, from moments taken on the
    device (``slice`` other than None, the maximum-current reference slice,
    is not supported).  Returns (tws, p_array) like the reference.
    """
    if slice is not None:
        raise NotImplementedError("slice='Imax' is not supported by device tracking; use slice=None")
    processes = None
    if navi is not None:
        if sc is None:
            processes = _navigator_processes(navi, lattice)
        unit_step = navi.unit_step if unit_step is None else unit_step
    if (sc is None and processes is None) or unit_step is None:
        raise ValueError("pass navi, or sc and unit_step")
    order = lattice_order(lattice) if order is None else int(order)
    job = DeviceTrack(lattice, sc, unit_step, p_array, graph=graph, order=order, processes=processes,
                      twiss=calc_tws, bounds=bounds).run()
    job.result(p_array)
    if calc_tws:
        return job.twiss_list(), p_array
    from .envelope import Twiss
    tws, L = [Twiss()], 0.
    for dz in job._step_dz:
        L += dz
        tw = Twiss()
        tw.s += L
        tws.append(tw)
    return tws, p_array
