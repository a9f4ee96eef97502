"""The uneven batch recorded into a CUDA graph (optifax_propagate_graph) and replayed.
Marked gpu.

A replay runs the same kernels on the same descriptors as optifax_propagate, so its
outputs and statistics equal the direct call's bit for bit, on every replay; the
inputs are read afresh by each replay (an input changed in place changes the next
replay's output exactly as a direct call with the new input would)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _specs():
    from optifax_gb300 import sweep
    insts = [sweep.Instance(1024, 0.15e-3, 29e-6, 1.0, 40e-15, 11),
             sweep.Instance(4096, 0.20e-3, 30e-6, 0.8, 100e-15, 13),
             sweep.Instance(8192, 0.05e-3, 28e-6, 3.0, 150e-15, 14),
             sweep.Instance(16384, 0.03e-3, 31e-6, 2.0, 150e-15, 17),
             sweep.Instance(1024, 0.30e-3, 32e-6, 2.0, 40e-15, 15)]
    return sweep.to_specs([sweep.build_inputs(i) for i in insts])


def test_graph_replays_equal_the_direct_call():
    from optifax_gb300 import solver as sv
    direct_specs = _specs()
    outs, stats = sv.propagate(direct_specs)
    torch.cuda.synchronize()
    ref = [o.cpu().numpy() for o in outs]
    ref_stats = sv.decode_stats(stats)
    specs = _specs()
    g = sv.propagate_graph(specs)
    assert g.kernels >= 2                                  # one grid per (cta_points, cluster) shape
    for _ in range(2):
        for o in g.outputs:
            o.zero_()
        g.launch()
        torch.cuda.synchronize()
        for o, r in zip(g.outputs, ref):
            assert np.array_equal(o.cpu().numpy(), r)
        assert sv.decode_stats(g.stats) == ref_stats
    g.close()


def test_graph_reads_inputs_afresh():
    from optifax_gb300 import solver as sv
    specs = _specs()
    g = sv.propagate_graph(specs)
    g.launch()
    torch.cuda.synchronize()
    specs[1].E.mul_(0.5)                                   # new input, same buffer
    g.launch()
    torch.cuda.synchronize()
    direct = _specs()
    direct[1].E.mul_(0.5)
    outs, _ = sv.propagate(direct)
    torch.cuda.synchronize()
    assert np.array_equal(g.outputs[1].cpu().numpy(), outs[1].cpu().numpy())
    g.close()
