"""Frame sharding over ranks + engstore merge, as world_size-2 gloo process groups on CPU.

Each rank accumulates its own frames (the CPU oracle stands in for the per-rank engine,
so the test needs no GPU); rank 0 merges through ermod_gb300.engstore (the library's
ermod_engstore_merge).  The merged, normalised distributions must equal one process
accumulating every frame."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


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
        w = synth.soln_small()
        w.params["estype"] = 2
    else:
        w = helpers.small_refs()
    return w


def _run_frames(w, frames):
    from oracle import oracle as O
    from tests import helpers
    topo, bins = helpers.build_inputs(w)
    orc = O.Oracle(w.params, topo, bins)
    for f in frames:
        pos, cell = w.frame(f)
        orc.frame(pos, cell)
        if w.mode == "soln":
            orc.placements([topo["nummol"]])
        else:
            pl = w.placements(f, 12)
            orc.placements(np.full(len(pl), topo["nummol"], np.int32), pl)
    return orc.accum()


def _rank(rank, world, port, mode, out):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from ermod_gb300 import engstore
    w = _work(mode)
    acc = _run_frames(w, [rank, rank + world])  # frames strided over ranks (plmode = 2)
    res = engstore.merge_distributed(acc, w.params["slttype"], w.params["wgtslf"], w.params["temp"])
    if rank == 0:
        np.savez(out, **{k: v for k, v in res.items() if v is not None})
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("mode", ["soln", "refs"])
def test_two_rank_merge_equals_single_process(tmp_path, mode, oracle, gpu_lib):
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
    # the self-energy offset is arbitrary; voffset +- kT log(avslf) is what engstore reports
    sign = -1.0 if w.params["slttype"] == 1 else 1.0
    T = w.params["temp"]
    np.testing.assert_allclose(merged["voffset"] + sign * T * np.log(merged["avslf"]),
                               ref["voffset"] + sign * T * np.log(ref["avslf"]), rtol=0, atol=1e-9)
    np.testing.assert_allclose(merged["minuv"], ref["minuv"])
    np.testing.assert_allclose(merged["maxuv"], ref["maxuv"])


def _bench_rank(rank, world, port, out):
    """One rank of bench.py's distributed branch: its own frames (bench.frames_of_rank)
    and the exchange (bench.merge_ranks, the product's engstore merge), with the oracle
    standing in for the per-rank GPU engine."""
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    w = _work("refs")
    acc = _run_frames(w, bench.frames_of_rank(rank, 2))
    res = bench.merge_ranks(acc, w)
    if rank == 0:
        np.savez(out, **{k: v for k, v in res.items() if v is not None})
    else:
        assert res is None
    dist.barrier()
    dist.destroy_process_group()


def test_bench_distributed_branch_merge(tmp_path, oracle, gpu_lib):
    out = str(tmp_path / "bench_merged.npz")
    port = _free_port()
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_bench_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(300)
        assert p.exitcode == 0
    import bench
    from ermod_gb300 import engstore
    assert bench.frames_of_rank(0, 2) == [0, 1] and bench.frames_of_rank(1, 2) == [2, 3]
    merged = dict(np.load(out))
    w = _work("refs")
    single = _run_frames(w, [0, 1, 2, 3])
    ref = engstore.merge([single], w.params["slttype"], w.params["wgtslf"], w.params["temp"])
    np.testing.assert_allclose(merged["edens"], ref["edens"], rtol=1e-9, atol=1e-14)
    np.testing.assert_allclose(merged["ecorr"], ref["ecorr"], rtol=1e-9, atol=1e-14)
    assert merged["engsmpl"] == ref["engsmpl"] == 4 * 12
