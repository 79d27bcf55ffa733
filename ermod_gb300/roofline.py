"""Algorithmic byte counts of the per-placement path (the roofline numerators).

Units: bytes per placement for a PME grid K1 x K2 x K3 with H = K1/2 + 1 half-complex
columns, FP32 grids (mixed path), N solvent sites and G placements per mol_energy CTA.
Each count is the least traffic the kernel's job needs: every value it must read or
write crosses HBM once.

  spectrum    writes the half spectrum engfac * S(k):            8 H K2 K3
  fft_c2r     reads it, writes the potential grid:               8 H K2 K3 + 4 K1 K2 K3
  gather      reads the potential grid once, plus the solvent
              site records (20 B) once per 4 placements:          4 K1 K2 K3 + 20 N / 4
  total                                                            16 H K2 K3 + 8 K1 K2 K3 + 5 N

The plain FP64 path doubles every grid term and adds the spread grid and the forward
transform (8 K^3 written by the spread, read by D2Z; 16 H K^2 written by D2Z).
"""
from __future__ import annotations

# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per placement of each mixed
# kernel, from one ncu --set full capture of a 256-placement launch of refs_large
# (33,000 waters, PME 96^3, order 4, 12-site solute).  At this batch the PME
# intermediate does not stay in L2, so these are close to the launch's full traffic;
# a launch of B placements moves about B times these bytes.
MEASURED_TRAFFIC_REFS_LARGE = {
    "spectrum": (8.3e6 + 865.7e6) / 256,  # pme_a: writes the half spectrum after the k3 transform
    "fft_c2r": (944.1e6 + 956.7e6) / 256,  # pme_b: reads it, writes the padded potential grid
    "gather": (1022.9e6 + 96.5e6) / 256,  # gather_tma: reads the grid (halo boxes) and site data
}

# From the same capture, per kernel: the issue and pipe use that bound it (percent of
# peak as ncu reports it) and its duration launched alone (us, one 256-placement launch,
# serialised and cold, so slower than inside the pipelined step).
MEASURED_PIPES_REFS_LARGE = {
    "spectrum": {"kernel": "pme_a_kernel<96>", "issue_active_pct": 62.7, "fma_pipe_pct": 40.8,
                 "alu_pipe_pct": 21.1, "fp64_pipe_pct": 0.5, "dram_pct": 15.3, "standalone_us": 720.9},
    "fft_c2r": {"kernel": "pme_b_kernel<96>", "issue_active_pct": 44.9, "fma_pipe_pct": 22.1,
                "alu_pipe_pct": 25.5, "fp64_pipe_pct": 0.0, "dram_pct": 34.8, "standalone_us": 688.9},
    "gather": {"kernel": "gather_tma_kernel<4>", "issue_active_pct": 28.2, "fma_pipe_pct": 18.3,
               "alu_pipe_pct": 4.7, "fp64_pipe_pct": 0.0, "dram_pct": 32.2, "standalone_us": 438.8},
}
PIPES_SOURCE = "profiles/kernels_refs_large_batch256.md"


def grid_terms(K1: int, K2: int, K3: int):
    H = K1 // 2 + 1
    return H * K2 * K3, K1 * K2 * K3


def bytes_per_placement(K1: int, K2: int, K3: int, nsite: int, G: int = 8) -> dict:
    nh, nr = grid_terms(K1, K2, K3)
    d = {
        "spectrum": 8.0 * nh,
        "fft_c2r": 8.0 * nh + 4.0 * nr,
        "gather": 4.0 * nr + 20.0 * nsite / 4,
    }
    d["total"] = sum(d.values())
    return d


def bytes_per_placement_fp64(K1: int, K2: int, K3: int, nsite: int) -> dict:
    nh, nr = grid_terms(K1, K2, K3)
    d = {
        "spectrum": 8.0 * nr + 8.0 * nr + 16.0 * nh + 2 * 16.0 * nh,  # spread, D2Z, influence
        "fft_c2r": 16.0 * nh + 8.0 * nr,
        "mol_energy": 8.0 * nr + (24 + 96 + 8 + 8) * nsite,
    }
    d["total"] = sum(d.values())
    return d
