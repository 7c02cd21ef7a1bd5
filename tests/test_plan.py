"""The run planner (mwf_describe_run, host only) against the batched kernels' compile-time bounds.

The FP32 batched kernels are instantiated for every line count (z pass) and column count (x
passes) an item can hold at their CTAs per SM, and reject items beyond those counts on the
device.  These tests restate the shared-memory formulas of mwf_zbatch.cuh / mwf_xbatch.cuh and
the per-SM budget of mwf_launch.h, and check that the planner only picks tilings the kernels
were built for, with the launch sizes they use.
"""
import numpy as np
import pytest

import mwf_gb300 as mwf
import bench

SMEM_PER_SM = 233472            # bytes of shared memory per SM usable by CTAs


def budget(blocks):
    return SMEM_PER_SM if blocks <= 1 else SMEM_PER_SM // blocks - 1024


def pad_elems(n):               # xb_pad_elems
    return (n + (n >> 4) + 2) & ~1


def zb_smem(K0, Q, L):          # zb_smem_bytes
    KK = 3 * K0 - 1
    ntr = (KK + 1) // 2 + KK
    n = 3 * ntr * L * Q
    return 16 * ((n + (n >> 4) + 2) & ~1)


def zb_minb(K0, Q):
    return 2 if zb_smem(K0, Q, 1) <= budget(2) else 1


def zb_lmax(K0, Q):
    L = 1
    while zb_smem(K0, Q, L + 1) <= budget(zb_minb(K0, Q)):
        L += 1
    return L


def xbf_smem(MM, nb):
    return 8 * (2 * pad_elems(6 * nb * MM) + 2 * nb * (2 * MM - 1))


def xbi_smem(MM, nb):
    return 16 * pad_elems(9 * nb * MM)


def nbmax(smem, MM, blocks):
    nb = 1
    while nb < 8 and smem(MM, nb + 1) <= budget(blocks):
        nb += 1
    return nb


BATCHED = [32, 48, 64, 96, 128, 192, 256]


@pytest.mark.parametrize("K0", [4, 6])
@pytest.mark.parametrize("N", BATCHED)
def test_batched_plans_stay_within_the_compiled_bounds(K0, N):
    p = mwf.RunParams(K0=K0, MM=N, NN=N, alpha=0.2, gamma=0.2, precision="fp32")
    if K0 == 6 and zb_smem(K0, N, 1) > budget(1):
        # no batched z pass at this size: the run-time-plan kernel takes it
        assert mwf.describe_run(p)["batched_z"] == 0
        return
    d = mwf.describe_run(p)
    KK, X = 3 * K0 - 1, 3 * N
    assert d["batched_x"] == 1 and d["batched_z"] == 1
    # z pass
    assert d["z_ctas_per_sm"] == zb_minb(K0, N)
    assert 1 <= d["z_lines"] <= zb_lmax(K0, N)
    assert d["z_smem"] == zb_smem(K0, N, d["z_lines"]) <= budget(d["z_ctas_per_sm"])
    assert d["z_items"] == -(-X // d["z_lines"])
    # x forward: three CTAs per SM, items of one wall-normal mode k
    assert d["xf_ctas_per_sm"] == 3
    assert 1 <= d["xf_cols"] <= min(nbmax(xbf_smem, N, 3), N)
    assert d["xf_smem"] == xbf_smem(N, d["xf_cols"]) <= budget(3)
    assert d["xf_items"] == -(-N // d["xf_cols"]) * K0
    # x inverse: four CTAs per SM
    assert d["xi_ctas_per_sm"] == 4
    assert 1 <= d["xi_cols"] <= min(nbmax(xbi_smem, N, 4), N)
    assert d["xi_smem"] == xbi_smem(N, d["xi_cols"]) <= budget(4)
    assert d["xi_items"] == -(-N // d["xi_cols"]) * K0
    # the planner takes the widest item that fits
    assert d["xf_cols"] == min(nbmax(xbf_smem, N, 3), N)
    assert d["xi_cols"] == min(nbmax(xbi_smem, N, 4), N)
    assert d["z_lines"] == min(zb_lmax(K0, N), X)


def test_ragged_column_blocks_and_uneven_sizes():
    # MM != NN, and NN not a multiple of the column count: the last block is narrower, which the
    # kernels' run-time dispatch over column counts covers
    d = mwf.describe_run(mwf.RunParams(K0=4, MM=96, NN=96, alpha=0.2, gamma=0.3, precision="fp32"))
    assert d["batched_x"] == 1 and d["batched_z"] == 1
    assert 96 % d["xf_cols"] != 0                       # five columns: a last block of one
    assert d["xf_items"] == -(-96 // d["xf_cols"]) * 4
    d = mwf.describe_run(mwf.RunParams(K0=4, MM=128, NN=96, alpha=0.2, gamma=0.3, precision="fp32"))
    assert d["batched_x"] == 1 and d["batched_z"] == 1
    assert d["xi_items"] == -(-96 // d["xi_cols"]) * 4
    assert d["z_items"] == -(-384 // d["z_lines"])
    assert d["z_smem"] == zb_smem(4, 96, d["z_lines"])   # the z line length is NN


def test_other_runs_take_the_run_time_plan_kernels():
    fp64 = mwf.describe_run(mwf.RunParams(K0=6, MM=512, NN=512, alpha=0.1, gamma=0.1))
    assert fp64["batched_x"] == 0 and fp64["batched_z"] == 0
    assert fp64["xf_ctas_per_sm"] == fp64["z_ctas_per_sm"] == fp64["xi_ctas_per_sm"] == 0
    # FP64: two fields (f, d/dx f) of KK per column block, three z partials per line block
    KK, X = 17, 1536
    assert fp64["xf_items"] == -(-512 // fp64["xf_cols"]) * 2 * KK
    assert fp64["z_items"] == -(-X // fp64["z_lines"]) * 3
    # an FP32 size without compile-time plans, and radix caps, select the same kernels
    odd = mwf.describe_run(mwf.RunParams(K0=4, MM=27, NN=36, alpha=0.2, gamma=0.2, precision="fp32"))
    assert odd["batched_x"] == 0 and odd["batched_z"] == 0
    capped = mwf.describe_run(mwf.RunParams(K0=4, MM=64, NN=64, alpha=0.2, gamma=0.2, precision="fp32",
                                            x_radix=8, z_radix=8))
    assert capped["batched_x"] == 0 and capped["batched_z"] == 0
    assert capped["z_items"] == -(-192 // capped["z_lines"])      # FP32 sums the three partials


def test_knobs_beyond_the_compiled_bounds_are_rejected():
    p = mwf.RunParams(K0=4, MM=128, NN=128, alpha=0.2, gamma=0.2, precision="fp32")
    with pytest.raises(mwf.MwfError):
        mwf.describe_run(p.with_(z_lines=zb_lmax(4, 128) + 1))
    with pytest.raises(mwf.MwfError):
        mwf.describe_run(p.with_(xi_cols=nbmax(xbi_smem, 128, 4) + 1))
    d = mwf.describe_run(p.with_(xf_cols=2, xi_cols=1))
    assert d["xf_cols"] == 2 and d["xi_cols"] == 1
    with pytest.raises(mwf.MwfError):
        mwf.describe_run(mwf.RunParams(K0=4, MM=35, NN=32, alpha=0.2, gamma=0.2))


def test_the_fp32_ensemble_workload_is_fully_batched():
    runs, _ = bench.workload_params("ensemble512-fp32")
    plans = [mwf.describe_run(p) for p in runs]
    assert all(d["batched_x"] and d["batched_z"] for d in plans)
    # one launch per pass and grid size: the step's fifteen launches
    sizes = {(p.MM, p.NN) for p in runs}
    assert len(sizes) == 5
    assert np.all([d["z_ctas_per_sm"] == 2 for d in plans])
