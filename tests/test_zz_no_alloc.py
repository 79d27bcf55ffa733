"""ermod_ecorr_add_noalloc against ermod_placements' own ecorr (marked gpu).

The engine's ecorr for unit-weight REFS placements with per-placement solute weights
is sum_p w_p h_p h_p^T, with h_p the histogram of placement p's energies.  The same
histograms, built on the host from the engine's uvengy, go through the no-allocation
entry point twice in a row (its fixed scratch is reused), once more with the device's
free memory read before and after (a warmed call allocates nothing), and once split in
two calls that accumulate into one matrix.  Sums run over placements in the same order as the
engine's, so the tolerance is a few ulps.
"""
import numpy as np
import pytest

from tests import helpers

pytestmark = pytest.mark.gpu


def _bind(L):
    from ermod_gb300 import _lib
    return L.ermod_ecorr_add_noalloc, _lib


def test_ecorr_noalloc_matches_engine(gpu_lib):
    import torch
    from ermod_gb300.engproc import EnergyRepresentation
    f, _lib = _bind(gpu_lib)
    w = helpers.small_refs(wgtslf=0)
    w.params["estype"] = 1
    topo, bins = helpers.build_inputs(w)
    eng = EnergyRepresentation(w.params, topo, bins, precision="mixed", count_mirror=True, batch=16)
    pos, cell = w.frame(0)
    pl = w.placements(0, 40)
    n = len(pl)
    tag = np.full(n, topo["nummol"], np.int32)
    sws = np.random.default_rng(5).uniform(0.5, 2.0, n)
    eng.frame(pos, cell)
    rg = eng.placements(tag, pl, stat_weight_solute=sws, want_uvengy=True)
    ref = eng.accum(with_count=True)
    eng.close()
    edges = bins["uvcrd"]
    ermax = len(edges)
    hist = np.stack([helpers.histogram(u, edges) for u in rg["uvengy"][:, 1:]]).astype(np.int32)
    assert hist.shape == (n, ermax)
    # the weights the engine used: stat_weight_system (1) x stat_weight_solute
    np.testing.assert_allclose(ref["edens"], (sws[:, None] * hist).sum(0), rtol=1e-12)

    dev = torch.device("cuda", 0)
    d_hist = torch.from_numpy(hist).to(dev)
    d_w = torch.from_numpy(sws).to(dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    ref_ecorr = ref["ecorr"].reshape(ermax, ermax)
    ref_count = ref["ecorr_count"].reshape(ermax, ermax)
    for call in range(2):  # the shared scratch is reused by the second call
        ecorr = torch.zeros((ermax, ermax), dtype=torch.float64, device=dev)
        count = torch.zeros((ermax, ermax), dtype=torch.int64, device=dev)
        st = f(d_hist.data_ptr(), d_w.data_ptr(), n, ermax, ecorr.data_ptr(), count.data_ptr(), stream)
        assert st == _lib.OK, gpu_lib.ermod_last_error_string()
        torch.cuda.synchronize(dev)
        np.testing.assert_allclose(ecorr.cpu().numpy(), ref_ecorr, rtol=1e-13, atol=0, err_msg=f"call {call}")
        np.testing.assert_array_equal(count.cpu().numpy(), ref_count)
    # a warmed call allocates nothing: the device's free memory (cudaMemGetInfo) is the
    # same before and after it
    ecorr.zero_()
    count.zero_()
    torch.cuda.synchronize(dev)
    free0, _ = torch.cuda.mem_get_info(dev)
    st = f(d_hist.data_ptr(), d_w.data_ptr(), n, ermax, ecorr.data_ptr(), count.data_ptr(), stream)
    assert st == _lib.OK
    torch.cuda.synchronize(dev)
    free1, _ = torch.cuda.mem_get_info(dev)
    assert free1 == free0, f"free device memory changed by {free0 - free1} bytes"
    np.testing.assert_array_equal(count.cpu().numpy(), ref_count)
    # two calls accumulating into one matrix, without the count mirror
    ecorr = torch.zeros((ermax, ermax), dtype=torch.float64, device=dev)
    h = n // 2
    for lo, hi in ((0, h), (h, n)):
        st = f(d_hist[lo:hi].data_ptr(), d_w[lo:hi].data_ptr(), hi - lo, ermax, ecorr.data_ptr(), None, stream)
        assert st == _lib.OK
    torch.cuda.synchronize(dev)
    np.testing.assert_allclose(ecorr.cpu().numpy(), ref_ecorr, rtol=1e-13, atol=0)


def test_ecorr_noalloc_rejects_sizes_beyond_its_scratch(gpu_lib):
    import torch
    f, _lib = _bind(gpu_lib)
    dev = torch.device("cuda", 0)
    one = torch.zeros(1, dtype=torch.float64, device=dev)
    ptr = one.data_ptr()
    for nplace, ermax in ((4097, 10), (10, 8193), (1024, 1025)):
        assert f(ptr, ptr, nplace, ermax, ptr, None, None) == _lib.E_PARAM
        assert b"scratch" in gpu_lib.ermod_last_error_string()
    assert f(ptr, ptr, 0, 10, ptr, None, None) == _lib.OK
