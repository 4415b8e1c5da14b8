"""Adapter giving the CPU oracle the state interface used by goldens.DebugRecorder
and refloop.run_reference_loop (test infrastructure)."""
import numpy as np

import oracle as O


class OracleRun:
    def __init__(self, settings, particle_init=None, restart_files=None, forwarded_init=None):
        self.s = settings
        self.o = O.EulerOracle(settings.oracle_config())
        self.particle_init = particle_init or {}
        self.forwarded_init = forwarded_init or {}
        self.restart_files = restart_files
        self.loaded_maps = None

    # stepper interface
    def init(self):
        for i, pos in self.particle_init.items():
            self.o.set_particles(i, pos)
        for i, pos in self.forwarded_init.items():
            self.o.set_forwarded_particles(i, pos)
        if self.s.restart_time != 0:
            # the restart branch of the driver reads the stored state instead of
            # building the Lagrange history (cmm-euler2d.cu:520-685)
            self.loaded_maps = self.o.restart(self.s.restart_time, self.restart_files)
        else:
            self.o.init()

    def step(self, dt_now):
        rc, e, r = self.o.step(dt_now)
        gap = (self.o.loop_ctr() - 1) - self.o.old_ctr()
        return rc, e, r, gap, self.o.map_count()

    # state interface
    def grid(self, k):
        g = self.o.grid(k)
        return (g.N, g.hx, g.hy)

    def chix(self):
        return self.o.chix()

    def chiy(self):
        return self.o.chiy()

    def psi(self):
        return self.o.psi()

    def vort(self):
        return self.o.vort()

    def particles(self, i):
        return self.o.particles(i)

    def particle_velocity(self, i):
        return self.o.particle_velocity(i)

    def energy(self):
        return self.o.energy()

    def enstrophy(self):
        return self.o.enstrophy()

    def palinstrophy(self):
        return self.o.palinstrophy()

    def max_vorticity(self):
        return self.o.max_vorticity()

    def vlasov_mesure(self):
        return self.o.vlasov_mesure()

    def sample(self, n, scalar_num):
        return self.o.sample(n, scalar_num)

    def zoom(self, n, bounds, scalar_num):
        return self.o.zoom(n, bounds, scalar_num)

    def chix_f(self):
        return self.o.chix_f()

    def chiy_f(self):
        return self.o.chiy_f()

    def forward_monitors(self):
        return self.o.forward_monitors()

    def forward_sample(self, n, bounds):
        return self.o.forward_sample(n, bounds)

