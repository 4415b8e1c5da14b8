"""Golden-fixture helpers shared by the CPU (oracle) and GPU (product) tests.

`reference_goldens.json` holds the reference's own golden monitoring series
(see tests/golden/make_golden.py).  `DebugRecorder` produces the same series
from any simulation state using the reference's writer semantics
(src/ui/cmm-io.cu:295-437 for which variables are written,
src/numerical/cmm-mesure.cu:217-249 for the statistics).
"""
import json
import os

import re

import numpy as np

from refloop import save_instant

HERE = os.path.dirname(os.path.abspath(__file__))
_G = None


def goldens():
    global _G
    if _G is None:
        with open(os.path.join(HERE, "golden", "reference_goldens.json")) as f:
            _G = json.load(f)
    return _G


def stats_grid(v, hx, hy):
    v = np.asarray(v, dtype=np.float64)
    return [float(v.min()), float(v.max()), hx * hy * max(0.0, float(v.max())), hx * hy * float(v.sum())]


def stats_raw(v):
    v = np.asarray(v, dtype=np.float64)
    return [float(v.min()), float(v.max()), max(0.0, float(v.max())) / v.size, float(v.sum()) / v.size]


def _has(var, *keys):
    return any(k in var for k in keys)


class DebugRecorder:
    """Collects Debug_globals / Mesure / monitoring series like the reference
    writes them at verbose=4.  `state` must provide grid(k) -> (N, hx, hy),
    chix(), chiy(), psi(), vort(), particles(i), particle_velocity(i),
    energy(), enstrophy(), palinstrophy(), max_vorticity()."""

    def __init__(self, settings, state):
        self.s = settings
        self.st = state
        self.series = {}
        self.forwarded = {}     # (t_now, set index) -> forwarded positions at a sample instant

    def _app(self, key, vals):
        self.series.setdefault(key, []).extend(vals)

    def _stat(self, name, vals):
        for suf, v in zip(("Min", "Max", "Avg", "L2"), vals):
            self._app("Debug_globals/%s_%s" % (name, suf), [v])

    def on_save(self, t_now, dt_now):
        s, st = self.s, self.st
        dt = s.dt
        var = ""
        fire = False
        for r in s.save_comp:
            if save_instant([r], t_now, dt_now, dt):
                fire = True
                var += r.var
        if fire:
            all_ = "All" in var
            gc, gp = st.grid(0), st.grid(2)
            if _has(var, "Vorticity", "W", "Stream", "Psi", "Map", "Chi", "Velocity", "U", "Dist", "F") or all_:
                self._app("Debug_globals/Time_s", [t_now])
                saved_any = True
            else:
                saved_any = False
            if _has(var, "Vorticity", "W") or all_:
                self._stat("Vorticity_W_coarse", stats_grid(st.vort(), gc[1], gc[2]))
            if _has(var, "Dist", "F") or all_:
                self._stat("Distribution_coarse", stats_grid(st.vort(), gc[1], gc[2]))
            psi = None
            if _has(var, "Stream", "Psi") or all_:
                psi = st.psi()
                self._stat("Stream_function_Psi_psi", stats_grid(psi[:gp[0]], gp[1], gp[2]))
            if _has(var, "Stream_H", "Psi_H") or all_:
                psi = st.psi() if psi is None else psi
                self._stat("Stream_function_Psi_H_psi", stats_raw(psi[:4 * gp[0]]))
            if _has(var, "Velocity", "U") or all_:
                psi = st.psi() if psi is None else psi
                self._stat("Velocity_UX_psi", stats_grid(psi[gp[0]:2 * gp[0]], gp[1], gp[2]))
                self._stat("Velocity_UY_psi", stats_grid(psi[2 * gp[0]:3 * gp[0]], gp[1], gp[2]))
            if _has(var, "Map_b", "Chi_b") or all_:
                self._stat("Map_ChiX_coarse", stats_grid(st.chix()[:gc[0]], gc[1], gc[2]))
                self._stat("Map_ChiY_coarse", stats_grid(st.chiy()[:gc[0]], gc[1], gc[2]))
            if _has(var, "Map_H", "Chi_H") or all_:
                self._stat("Map_ChiX_H_coarse", stats_raw(st.chix()))
                self._stat("Map_ChiY_H_coarse", stats_raw(st.chiy()))
            if s.forward_map and (_has(var, "Map_f", "Chi_f") or all_):
                self._stat("Map_ChiX_f_coarse", stats_grid(st.chix_f()[:gc[0]], gc[1], gc[2]))
                self._stat("Map_ChiY_f_coarse", stats_grid(st.chiy_f()[:gc[0]], gc[1], gc[2]))
            if s.forward_map and (_has(var, "Map_f_H", "Chi_f_H") or all_):
                self._stat("Map_ChiX_f_H_coarse", stats_raw(st.chix_f()))
                self._stat("Map_ChiY_f_H_coarse", stats_raw(st.chiy_f()))
            if "PartA_" in var or all_:
                if not saved_any:
                    self._app("Debug_globals/Time_s", [t_now])
            for i, p in enumerate(s.particles_advected):
                if ("PartA_%02d" % (i + 1)) in var or all_:
                    self._stat("Particles_advected_pos_P%02d" % (i + 1), stats_raw(st.particles(i)))
                if ("PartA_Vel_%02d" % (i + 1)) in var or all_:
                    # inertial sets: their velocity state; tracers: (psi_x, psi_y) sampled there
                    self._stat("Particles_advected_vel_U%02d" % (i + 1), stats_raw(st.particle_velocity(i)))
        # compute_conservation_targets (cmm-simulation-host.cu:615-698)
        if save_instant(s.save_comp, t_now, dt_now, dt, need_conv=True) and s.simulation_type_num == 2:
            m = st.vlasov_mesure()
            self._app("Mesure/Time_s", [t_now])
            for k in ("Etot", "Ekin", "Epot", "Mass", "Momentum", "Emode1", "Emode2", "Emode3", "Emode4"):
                self._app("Mesure/" + k, [m[k]])
        elif save_instant(s.save_comp, t_now, dt_now, dt, need_conv=True):
            self._app("Mesure/Time_s", [t_now])
            self._app("Mesure/Energy", [st.energy()])
            self._app("Mesure/Enstrophy", [st.enstrophy()])
            self._app("Mesure/Palinstrophy", [st.palinstrophy()])
            self._app("Mesure/Max_vorticity", [st.max_vorticity()])

        # sample_compute_and_write (cmm-simulation-host.cu:706-893), backward-map part
        if s.simulation_type_num != 2:
            for r in s.save_sample:
                if not save_instant([r], t_now, dt_now, dt):
                    continue
                n, var = r.grid, r.var
                all_ = "All" in var
                b = s.domain_bounds
                hx, hy = (b[1] - b[0]) / n, (b[3] - b[2]) / n
                self._app("Debug_globals/Time_s_%d" % n, [t_now])
                if s.forward_map and (_has(var, "Map_f", "Chi_f") or all_ or s.particles_forwarded):
                    fx, fy, parts = st.forward_sample(n, b[:4])
                    if _has(var, "Map_f", "Chi_f") or all_:
                        self._stat("Map_ChiX_f_%d" % n, stats_grid(fx, hx, hy))
                        self._stat("Map_ChiY_f_%d" % n, stats_grid(fy, hx, hy))
                    for i, p in enumerate(parts):
                        self.forwarded[(t_now, i)] = p
                planes, mes = st.sample(n, s.scalar_num)

                def stat(name):
                    self._stat("%s_%d" % (name, n), stats_grid(planes[name], hx, hy))
                if _has(var, "Map_b", "Chi_b") or all_:
                    stat("Map_ChiX")
                    stat("Map_ChiY")
                if _has(var, "Scalar", "Theta") or all_:
                    stat("Scalar_Theta")
                    self._app("Mesure/Scalar_integral_%d" % n, [mes["Scalar_integral"]])
                if _has(var, "Vorticity", "W", "F") or all_:
                    stat("Vorticity_W")
                if _has(var, "Laplacian_W") or all_:
                    stat("Laplacian_W")
                if _has(var, "Grad_W") or all_:
                    stat("GradX_W")
                    stat("GradY_W")
                if _has(var, "Stream", "Psi") or all_:
                    stat("Stream_function_Psi")
                if _has(var, "Velocity", "U") or all_:
                    stat("Velocity_UX")
                    stat("Velocity_UY")
                self._app("Mesure/Time_s_%d" % n, [t_now])
                for k in ("Energy", "Enstrophy", "Palinstrophy", "Max_vorticity"):
                    self._app("Mesure/%s_%d" % (k, n), [mes[k]])

        # compute_zoom (cmm-simulation-host.cu:1039-1201), backward-map part: statistics with
        # the spacing of an n x n grid over the whole domain (the zoom variable's own grid)
        if s.simulation_type_num != 2:
            for iz, r in enumerate(s.save_zoom):
                if not save_instant([r], t_now, dt_now, dt):
                    continue
                n, var = r.grid, r.var
                all_ = "All" in var
                b = s.domain_bounds
                hx, hy = (b[1] - b[0]) / n, (b[3] - b[2]) / n
                self._app("Debug_globals/Time_s_%d_Zoom_%d" % (n, iz + 1), [t_now])
                wx, wy = r.width_x / 2.0, r.width_y / 2.0
                for rep in range(r.rep):
                    win = (r.pos_x - wx, r.pos_x + wx, r.pos_y - wy, r.pos_y + wy)
                    planes = st.zoom(n, win, s.scalar_num)
                    if s.forward_map and (_has(var, "Map_f", "Chi_f") or all_):
                        planes["Map_ChiX_f"], planes["Map_ChiY_f"], _ = st.forward_sample(n, win)

                    def stat(name):
                        self._stat("%s_%d_Zoom_%d_rep_%d" % (name, n, iz + 1, rep), stats_grid(planes[name], hx, hy))
                    if s.forward_map and (_has(var, "Map_f", "Chi_f") or all_):
                        stat("Map_ChiX_f")
                        stat("Map_ChiY_f")
                    if _has(var, "Map_b", "Chi_b") or all_:
                        stat("Map_ChiX")
                        stat("Map_ChiY")
                    if _has(var, "Scalar", "Theta") or all_:
                        stat("Scalar_Theta")
                    if _has(var, "Vorticity", "W") or all_:
                        stat("Vorticity_W")
                    if _has(var, "Dist", "F") or all_:
                        stat("Distribution")
                    if _has(var, "Stream", "Psi") or all_:
                        stat("Stream_function_Psi")
                    wx *= r.rep_fac
                    wy *= r.rep_fac

    def on_step(self, loop_ctr, t, e_inc, gap, maps):
        self._app("Time_s", [t])
        self._app("Error_incompressibility", [e_inc])
        if self.s.forward_map:
            ef, ev = self.st.forward_monitors()
            self._app("Error_incompressibility_forward", [ef])
            self._app("Error_invertibility", [ev])
        self._app("Map_gaps", [float(gap)])
        self._app("Map_counter", [float(maps)])


def compare_series(ours, gold, keys, rtol):
    """Return list of (key, worst scaled error) and failures.  Each golden value
    g is compared to ours o as |o-g| <= rtol*scale, scale being the magnitude of
    the data the statistic summarises (so sums of zero-mean fields compare on
    the magnitude of their terms, not on their near-zero total)."""
    worst = []
    fails = []
    for k in keys:
        if k not in gold:
            continue
        g = np.asarray(gold[k], dtype=np.float64)
        o = np.asarray(ours.get(k, []), dtype=np.float64)
        if o.shape != g.shape:
            fails.append((k, "length %d vs golden %d" % (o.size, g.size)))
            continue
        base = k.rsplit("_", 1)[0] if k.startswith("Debug_globals/") else k
        if k.startswith("Debug_globals/") and k.rsplit("_", 1)[-1] in ("Min", "Max", "Avg", "L2"):
            mn = np.abs(np.asarray(gold.get(base + "_Min", g)))
            mx = np.abs(np.asarray(gold.get(base + "_Max", g)))
            mag = np.maximum(mn, mx)
            if k.endswith("_L2") or k.endswith("_Avg"):
                # grid form multiplies by hx*hy*N ~ area; raw form divides by N
                area_scale = np.maximum(np.abs(g), mag * (4 * np.pi ** 2 if "Particles" not in k and "_H_" not in k else 1.0))
                scale = np.maximum(area_scale, 1e-300)
            else:
                scale = np.maximum(mag, 1e-300)
        elif k in ("Error_incompressibility", "Error_incompressibility_forward", "Error_invertibility"):
            # |1 - det grad X| with det ~ 1, |x - X_b(X_f(x))| with x ~ 1: deviations of O(1)
            # quantities, absolute on their scale
            scale = np.ones_like(g)
        else:
            scale = np.maximum(np.abs(g), 1e-300)
        err = np.abs(o - g) / scale
        m = re.match(r"Debug_globals/Map_Chi[XY](?:_f)?_(\d+)(?:_Zoom_\d+_rep_\d+)?_(Min|Max|L2|Avg)$", k)
        if m:
            # positions of a sampled (backward or forward) map are wrapped into [0, W): a point
            # whose composed position lies within rounding of the boundary lands at ~0 in one
            # implementation and at ~W in another (for 4_nodes the line y = 0 is invariant, so
            # such points always exist).  Accept whole periods of such points.
            n, stat = int(m.group(1)), m.group(2)
            W, near = 2 * np.pi, 1e-10
            hh = (W / n) ** 2     # statistics use the spacing of the n x n grid over the domain
            if stat == "L2":
                per = W * hh
                kk = np.round((o - g) / per)
                err = np.where(np.abs(kk) <= 4, np.abs(o - g - kk * per) / scale, err)
            elif stat == "Min":
                err = np.where(np.minimum(o, g) < near * W, 0.0, err)
            elif stat == "Max":
                err = np.where(np.maximum(o, g) > W * (1 - near), 0.0, err)
            else:   # Avg = hx hy max(0, max)
                err = np.where(np.maximum(o, g) > hh * W * (1 - near), 0.0, err)
        m = re.match(r"Debug_globals/Particles_advected_pos_P\d+_(Min|Max|L2|Avg)$", k)
        if m and base + "_Avg" in gold and base + "_Max" in gold:
            # particle positions are wrapped into [0, W) the same way: a particle on a line the
            # flow leaves invariant (y = 0 for 4_nodes) sits within rounding of the boundary at
            # every step and lands at ~0 in one implementation and at ~W in another.  Accept
            # whole periods of such particles.  Raw form over n values: Avg = max(0, max) / n,
            # L2 = sum / n, so n = Max / Avg.
            stat = m.group(1)
            W, near = 2 * np.pi, 1e-10
            gmax, gavg = np.asarray(gold[base + "_Max"], dtype=np.float64), np.asarray(gold[base + "_Avg"], dtype=np.float64)
            n = np.where(gavg > 0, np.round(gmax / np.where(gavg > 0, gavg, 1.0)), 0.0)
            if stat == "L2":
                per = np.where(n > 0, W / np.maximum(n, 1.0), np.inf)
                kk = np.round((o - g) / per)
                err = np.where((np.abs(kk) <= 8) & (n > 0), np.abs(o - g - kk * per) / scale, err)
            elif stat == "Min":
                err = np.where(np.minimum(o, g) < near * W, 0.0, err)
            elif stat == "Max":
                err = np.where(np.maximum(o, g) > W * (1 - near), 0.0, err)
            else:
                err = np.where(np.maximum(o, g) * n > W * (1 - near), 0.0, err)
        e = float(err.max()) if err.size else 0.0
        worst.append((k, e))
        if not np.all(err <= rtol):
            fails.append((k, e))
    return worst, fails
