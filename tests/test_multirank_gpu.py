"""Frame sharding over two ranks of the GPU engine itself (marked gpu).

Two processes (a world_size-2 gloo group, spawned) each run the mixed-precision engine on
the one GPU for their own frames (strided, the reference's plmode = 2) and merge through
ermod_gb300.engstore (ermod_engstore_merge).  Their kernels never wait on one another:
the one exchange is the host-side merge.  The merged, normalised distributions must equal
one engine accumulating every frame (to the rounding of the FP64 sums' order; counts
exactly)."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

pytestmark = pytest.mark.gpu


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _work(mode):
    from ermod_gb300 import synth
    from tests import helpers
    if mode == "soln":
        w = synth.soln_small(frames=4)
        w.params["estype"] = 2
    else:
        w = helpers.small_refs()
    return w


def _run_frames(w, frames):
    """The engine over the given frames (24 placements per frame in reference mode)."""
    from ermod_gb300.engproc import EnergyRepresentation
    from tests import helpers
    topo, bins = helpers.build_inputs(w)
    eng = EnergyRepresentation(w.params, topo, bins, precision="mixed", batch=8)
    for f in frames:
        eng.frame(*w.frame(f))
        if w.mode == "soln":
            eng.placements([topo["nummol"]])
        else:
            pl = w.placements(f, 24)
            eng.placements(np.full(len(pl), topo["nummol"], np.int32), pl)
    acc = eng.accum()
    eng.close()
    return acc


def _rank(rank, world, port, mode, out):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from ermod_gb300 import engstore
    w = _work(mode)
    acc = _run_frames(w, [rank, rank + world])
    res = engstore.merge_distributed(acc, w.params["slttype"], w.params["wgtslf"], w.params["temp"])
    if rank == 0:
        np.savez(out, **{k: v for k, v in res.items() if v is not None})
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("mode", ["soln", "refs"])
def test_two_engine_ranks_merge_equals_one_engine(tmp_path, mode, gpu_lib):
    out = str(tmp_path / "merged.npz")
    port = _free_port()
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_rank, args=(r, 2, port, mode, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(300)
        assert p.exitcode == 0
    merged = dict(np.load(out))
    from ermod_gb300 import engstore
    w = _work(mode)
    single = _run_frames(w, [0, 2, 1, 3])
    ref = engstore.merge([single], w.params["slttype"], w.params["wgtslf"], w.params["temp"])
    np.testing.assert_allclose(merged["edens"], ref["edens"], rtol=1e-9, atol=1e-14)
    if mode == "refs":
        np.testing.assert_allclose(merged["ecorr"], ref["ecorr"], rtol=1e-9, atol=1e-14)
    assert merged["engsmpl"] == ref["engsmpl"]
    sign = -1.0 if w.params["slttype"] == 1 else 1.0
    T = w.params["temp"]
    np.testing.assert_allclose(merged["voffset"] + sign * T * np.log(merged["avslf"]),
                               ref["voffset"] + sign * T * np.log(ref["avslf"]), rtol=0, atol=1e-9)
    np.testing.assert_array_equal(merged["minuv"], ref["minuv"])
    np.testing.assert_array_equal(merged["maxuv"], ref["maxuv"])
