"""Equilibration: adaptation of the maximum steps during nequil (Updater::simulate's
adjustment block, scOOP/mc/updater.cpp:238-253, with optimizeStep / optimizeRot,
updater.cpp:395-464) and the equilibrate-then-produce sequence of main.cpp:270-297.

The adjustment is restated here on the acceptance counts the GPU run records per particle
type; the library's adapted steps must follow the restatement exactly, over several
adjustments and for the box edge of an NPT run."""
import math
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


class Disp:
    """The reference's Disp record (statistics.h:53-66) and its two update rules."""

    def __init__(self, mx):
        self.mx, self.oldrmsd, self.oldmx = mx, 0.0, 0.0

    def optimize_step(self, acc, rej, hi, lo):
        ratio = acc / (acc + rej) if acc + rej > 0 else 0.0
        new = self.mx * ratio
        if self.oldrmsd > 0:
            if new < self.oldrmsd:
                if self.oldmx > 1:
                    self.mx /= 1.05
                    self.oldmx = 0.95
                else:
                    self.mx *= 1.05
                    self.oldmx = 1.05
            else:
                if self.oldmx > 1:
                    self.mx *= 1.05
                    self.oldmx = 1.05
                else:
                    self.mx /= 1.05
                    self.oldmx = 0.95
        if new > 0:
            self.oldrmsd = new
        else:
            self.oldrmsd = 0.0
            self.mx /= 1.05
            self.oldmx = 0.95
        self.mx = min(max(self.mx, lo), hi)

    def optimize_rot(self, acc, rej, hi, lo):
        ratio = acc / (acc + rej) if acc + rej > 0 else 0.0
        new = self.mx * ratio
        if self.oldrmsd > 0:
            if new > self.oldrmsd:
                if self.oldmx > 1:
                    self.mx *= 0.99
                    self.oldmx *= 0.99
                else:
                    self.mx *= 1.01
                    self.oldmx *= 1.01
            else:
                if self.oldmx > 1:
                    self.mx *= 1.01
                    self.oldmx *= 1.01
                else:
                    self.mx *= 0.99
                    self.oldmx *= 0.99
        if new > 0:
            self.oldrmsd = new
        else:
            self.oldrmsd = 0.0
            self.mx *= 1.01
            self.oldmx = 1.01
        self.mx = min(max(self.mx, lo), hi)


def test_adjusted_steps_follow_the_reference_rule():
    from sc_gb300 import System, workloads

    s = System.from_text(*workloads.npt_cpsc_spa(400, seed=5))
    s0 = s.step_sizes()
    types = [1, 2]                      # CPSC (type 1) and SPA (type 2)
    trans = {t: Disp(s0.trans[t]) for t in types}
    rot = {t: Disp(s0.rot_cos[t]) for t in types}
    edge = Disp(s0.edge)
    moved = []
    for k in range(5):
        st = s.simulate(nsweeps=20, seed=11, check_every=0)
        c = s.step_sizes()
        for t in types:
            if c.acc_trans[t] + c.rej_trans[t] > 0:
                trans[t].optimize_step(c.acc_trans[t], c.rej_trans[t], 1.5, 0.0)
            if c.acc_rot[t] + c.rej_rot[t] > 0:
                rot[t].optimize_rot(c.acc_rot[t], c.rej_rot[t], 5.0, 0.01)
        assert c.acc_edge + c.rej_edge == st.acc_vol + st.rej_vol
        assert sum(c.acc_trans[t] for t in types) == st.acc_trans
        assert sum(c.acc_rot[t] + c.rej_rot[t] for t in types) == st.acc_rot + st.rej_rot
        edge.optimize_step(c.acc_edge, c.rej_edge, 1.0, 0.0)
        s.adjust_steps()
        a = s.step_sizes()
        for t in types:
            assert a.trans[t] == trans[t].mx, (k, t, a.trans[t], trans[t].mx)
            assert a.rot_cos[t] == rot[t].mx, (k, t)
        assert a.edge == edge.mx and a.adjustments == k + 1
        assert s.default_run().edge_mx == edge.mx       # later runs use the adapted edge range
        moved.append(a.trans[1])
    assert len(set(moved)) > 1                          # the steps did adapt
    # the spheres never rotate: their rotation record is untouched
    assert a.acc_rot[2] + a.rej_rot[2] == 0 and a.rot_cos[2] == s0.rot_cos[2]
    st = s.simulate(nsweeps=10, seed=12, check_every=0)
    exact = s.all_to_all()
    assert abs(st.energy - exact) <= 1e-9 * max(1.0, abs(exact))
    s.close()


def test_equilibration_then_production_writes_config_eq(tmp_path):
    """main.cpp:270-297 through the output loop: nequil/2 sweeps adjusting every `adjust`
    sweeps, nequil/2 without, config.eq, then the production run.  The same sequence done by
    hand (sc_simulate blocks and sc_adjust_steps) on an identical system and seed ends with
    the same steps and the same state."""
    from sc_gb300 import System, updater, workloads

    texts = workloads.nvt_psc(300, phi=0.15, seed=4)
    s = System.from_text(*texts)
    tot = updater.run(s, 40, report=20, directory=str(tmp_path), nequil=60, adjust=10, seed=3)
    assert tot["sweeps"] == 40 and tot["equilibration_sweeps"] == 60
    eq = (tmp_path / "config.eq").read_text().splitlines()
    assert len(eq) == 1 + s.n and len(eq[1].split()) == 11
    a = s.step_sizes()
    assert a.adjustments == 3
    last = (tmp_path / "config.last").read_text().splitlines()
    assert len(last) == 1 + s.n and last != eq
    h = System.from_text(*texts)
    for _ in range(3):
        h.simulate(nsweeps=10, seed=3, check_every=100)
        h.adjust_steps()
    h.simulate(nsweeps=30, seed=3, check_every=100)
    b = h.step_sizes()
    assert b.adjustments == 3 and list(b.trans) == list(a.trans) and list(b.rot_cos) == list(a.rot_cos)
    h.write_config(str(tmp_path / "by_hand.eq"))
    assert (tmp_path / "by_hand.eq").read_text().splitlines() == eq
    s.close()
    h.close()
