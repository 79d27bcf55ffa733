"""The intermediate-state extension (extensions/Intermediate/engproc.F90) on the GPU
against the oracle (marked gpu): solution mode over several frames, with a
reference-solvent density whose upper bins are empty so that some frames fall outside
the intermediate state and some inside."""
import numpy as np
import pytest

from ermod_gb300 import engstore
from tests import helpers

pytestmark = pytest.mark.gpu


def test_intermediate_state_matches_oracle(gpu_lib, oracle, tmp_path):
    from ermod_gb300 import synth
    from ermod_gb300.engproc import EnergyRepresentation
    w = synth.soln_small()
    topo, bins = helpers.build_inputs(w)
    edges = bins["uvcrd"]
    tag = [topo["nummol"]]
    orc = oracle.Oracle(w.params, topo, bins)
    frames = range(6)
    umax = []
    for f in frames:  # where the frames' most repulsive molecules fall
        pos, cell = w.frame(f)
        orc.frame(pos, cell)
        umax.append(orc.placements(tag)["uvengy"][0, 1:].max())
    cut = float(np.median(umax))
    assert min(umax) < cut < max(umax) or min(umax) < cut
    refs = np.where(edges[:len(edges)] > cut, 0.0, 1.0)  # bins above the cut are empty in the reference
    orc = oracle.Oracle(w.params, topo, bins)
    gpu = EnergyRepresentation(w.params, topo, bins, precision="mixed")
    orc.intermediate_enable(refs)
    gpu.intermediate_enable(refs)
    for f in frames:
        pos, cell = w.frame(f)
        orc.frame(pos, cell)
        orc.placements(tag)
        gpu.frame(pos, cell)
        gpu.placements(tag)
    ro, rg = orc.intermediate_get(), gpu.intermediate_get()
    assert 0 < ro["soln_intm"] < ro["soln_total"]
    for k in ("soln_total", "soln_intm", "norm_intm"):
        np.testing.assert_allclose(rg[k], ro[k], rtol=1e-12)
    np.testing.assert_allclose(rg["edintm"].sum(), ro["edintm"].sum(), rtol=1e-12)
    np.testing.assert_allclose(rg["uvintm"], ro["uvintm"], rtol=1e-6, atol=1e-3)
    paths = engstore.write_intermediate(str(tmp_path), rg, bins, w.params["temp"], 1, 1)
    assert sorted(p.split("/")[-1] for p in paths) == ["Prob_Result", "avint.tt", "engint.tt"]
    back = engstore.read_engdist(str(tmp_path / "engint.tt"))
    np.testing.assert_allclose(back, rg["edintm"] / rg["norm_intm"], rtol=1e-14)
    gpu.close()
