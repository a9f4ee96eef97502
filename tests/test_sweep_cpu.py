"""The uneven sweep's instances (config 3: 256 crystal passes, seed 2) follow their
stated distributions, and each instance's solver inputs are self-consistent."""
import numpy as np

from optifax_gb300 import physics as ph, sweep


def test_instances_cover_the_stated_ranges():
    insts = sweep.uneven_sweep_instances()
    assert len(insts) == 256
    assert insts == sweep.uneven_sweep_instances()                     # seeded
    assert insts != sweep.uneven_sweep_instances(seed=3)
    n = np.array([i.n_points for i in insts])
    assert set(n.tolist()) == {2 ** k for k in range(12, 17)}           # every size drawn
    assert np.all(np.bincount(np.log2(n).astype(int))[12:] > 256 // 5 // 2)
    for name, lo, hi in (("length", 0.5e-3, 10e-3), ("period", 28e-6, 32e-6), ("power", 0.5, 3.0),
                         ("tau", 100e-15, 300e-15)):
        v = np.array([getattr(i, name) for i in insts])
        assert v.min() >= lo and v.max() <= hi
        assert v.min() < lo + 0.1 * (hi - lo) and v.max() > hi - 0.1 * (hi - lo)
    assert len({i.seed for i in insts}) == 256                          # one noise stream each


def test_instance_inputs_share_one_sample_spacing():
    """A fixed dt of 6 ps / 2^13, so the window grows with N; one step per 0.1 um of crystal."""
    for inst in sweep.uneven_sweep_instances(n=6, seed=5):
        win, si, e = sweep.build_inputs(inst)
        assert abs(win.dt / sweep.DT - 1) < 1e-9                        # dt = t[1] - t[0] of the grid
        assert e.shape == (inst.n_points,) and np.all(np.isfinite(e))
        assert si.n_steps == ph.Crystal(inst.length, inst.period).n_steps == int(inst.length / 1e-7)
