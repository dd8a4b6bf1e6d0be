"""The physics-process plugin contract of Ocelot's Navigator.

Mirrors ``PhysProc`` (ocelot/cpbd/physics_proc.py:14-70): the attributes that
``ProcessTable.add_physics_proc`` assigns (ocelot/cpbd/navi.py:68-81) and the
``prepare`` / ``apply`` / ``finalize`` hooks that ``track()`` calls
(ocelot/cpbd/track.py:476-478, 498-499).  Navigator only duck-types these, so
a process derived from this class drops into an unchanged Navigator.
"""


class PhysProc:
    def __init__(self, step=1):
        self.step = step
        self.energy = None
        self.indx0 = None
        self.indx1 = None
        self.s_start = None
        self.s_stop = None
        self.start_elem = None
        self.end_elem = None
        self.z0 = None

    def check_step(self):
        # same test as physics_proc.py:37-39
        if not isinstance(self.step, (int, float)) and float(self.step).is_integer():
            raise ValueError(f'step must be an integer number, instead {self.step}')

    def prepare(self, lat):
        self.check_step()

    def apply(self, p_array, dz):
        pass

    def finalize(self, *args, **kwargs):
        pass
