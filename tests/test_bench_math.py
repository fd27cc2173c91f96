"""CPU: the roofline arithmetic of bench.py (algorithmic bytes of the FP64
steppers, the choice between the one-signal and the paired launch)."""

import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402

N, NNZ = 73313, 1085113     # the 40^3 two-compartment workload


def test_pair_bytes_reduce_to_single():
    """A pair whose second signal never iterates moves the single signal's bytes
    plus the second signal's per-step vector traffic (32 bytes per dof)."""
    its = np.array([[21, 19, 25, 18], [0, 0, 0, 0]])
    steps = its.shape[1]
    single = bench.alg_bytes_fp64(N, NNZ, steps, its[0].sum())
    assert bench.alg_bytes_fp64_pair(N, NNZ, its) == single + 32 * N * steps


def test_pair_bytes_share_the_matrix():
    """Two signals with equal counts: the matrix is read once per pair
    iteration, so the pair moves less than two single launches by exactly the
    matrix bytes of one signal's iterations and right-hand sides."""
    its = np.array([[20, 22, 24], [20, 22, 24]])
    steps, it = its.shape[1], int(its[0].sum())
    two = 2 * bench.alg_bytes_fp64(N, NNZ, steps, it)
    shared = (NNZ * 28 + 4 * N) * steps + (NNZ * 20 + 4 * N) * it
    assert bench.alg_bytes_fp64_pair(N, NNZ, its) == two - shared


def test_pair_bytes_follow_the_slower_signal():
    its = np.array([[10, 30], [30, 10]])
    matrix_iter = NNZ * 20 + 4 * N
    assert (bench.alg_bytes_fp64_pair(N, NNZ, its) - bench.alg_bytes_fp64_pair(N, NNZ, its * 0)
            == matrix_iter * 60 + 160 * N * 80)


def test_roofline_picks_the_launch_form():
    info = {"n_dofs": N, "nnz": NNZ}
    its = np.array([[20] * 270, [22] * 270])
    pair = bench.roofline_fp64(info, {"kernel_launches": 5, "stepper_ms": 400.0, "steps": 270,
                                      "total_iterations": int(its.sum())}, its, 6793.4, "test", None)
    assert pair["kernel"].startswith("k_step64_pair")
    assert pair["launch_ms"] == 400.0
    assert pair["bytes_per_launch"] == bench.alg_bytes_fp64_pair(N, NNZ, its)
    single = bench.roofline_fp64(info, {"kernel_launches": 6, "stepper_ms": 500.0, "steps": 270,
                                        "total_iterations": int(its.sum())}, its, 6793.4, "test", None)
    assert single["kernel"].startswith("k_step64 ")
    assert single["launch_ms"] == 250.0
    assert single["bytes_per_launch"] == bench.alg_bytes_fp64(N, NNZ, 270, its.sum() / 2)
    assert abs(pair["frac"] - pair["achieved"] / 6793.4) < 1e-12
    assert single["note"] == "no DRAM capture for this workload"
