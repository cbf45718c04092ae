"""Launch shapes of the fast kernels (nqcd_set_mapping, picked by the project
autotuner): every shape gives the same physics.

* Spin-boson: the block size does not change which lanes hold a trajectory,
  so results are bitwise those of the default; eight lanes per trajectory
  change only the order of the bath sums, so the population correlation
  agrees to FP32 rounding.
* Ring polymers: every lane group of a bead count gives the same
  state-resolved scattering within sampling error.
* Shapes outside the lists, and eight spin-boson lanes without Kahan
  accumulation, are refused.
"""
import numpy as np
import pytest

from nqcd_gb300 import _lib as L
from nqcd_gb300 import autotune
from nqcd_gb300 import configs as C
from nqcd_gb300 import workload as WL

pytestmark = pytest.mark.gpu


def run_sb(mapping, n=4096, nmodes=100, t1=4.0, dt=0.05, prec=L.PREC_FP32_KAHAN):
    w, c, r0, v0 = WL.spin_boson_inputs(n, nmodes)
    stride = 2
    eng = C.spinboson_fssh(L, w, c, n, nmodes, prec, save_stride=stride)
    try:
        if mapping:
            eng.set_mapping(mapping)
        eng.set_initial(np.ascontiguousarray(r0), np.ascontiguousarray(v0))
        pc = np.zeros((round(t1 / dt) // stride + 1) * 4)
        eng.run(0.0, t1, dt, 7, popcorr=pc)
        fin = eng.get_final(nmodes)
        return pc.reshape(-1, 4), fin
    finally:
        eng.close()


def test_spinboson_block_size_is_bitwise_neutral():
    base_pc, base = run_sb(None)
    for block in (64, 256):
        pc, fin = run_sb(dict(sb_block=block))
        np.testing.assert_array_equal(pc, base_pc)
        for key in ("r", "v", "state", "nhops"):
            np.testing.assert_array_equal(fin[key], base[key], err_msg=f"{key} block {block}")


def test_spinboson_eight_lanes_match_four():
    base_pc, base = run_sb(None)
    pc, fin = run_sb(dict(sb_lanes=8, sb_block=128))
    np.testing.assert_allclose(pc, base_pc, atol=2e-3)
    assert np.mean(fin["state"] == base["state"]) > 0.95
    np.testing.assert_allclose(fin["r"].mean(0), base["r"].mean(0), atol=2e-2 * np.abs(base["r"]).std())


def test_rpsh_lane_groups_give_the_same_scattering():
    n = 8192
    r0, v0, _, models = C.rpsh_inputs(n)
    for beads, cands in autotune.RP_LANES.items():
        nb = np.full(n, beads, np.int32)
        res = {}
        for lanes in cands:
            eng = C.rpsh_tully(L, n, L.PREC_FP32)
            try:
                eng.set_mapping(dict(rp_lanes={beads: lanes}))
                eng.set_initial(np.ascontiguousarray(r0), np.ascontiguousarray(v0), nbeads=nb)
                eng.set_trajectory_models(np.ascontiguousarray(models))
                sc = np.zeros(4)
                eng.run(0.0, 20000.0, 1.0, 5, scattering=sc)
                res[lanes] = sc
            finally:
                eng.close()
        ref = res[4]
        sig = np.sqrt(np.maximum(ref, 1.0 / n) * (1 - ref) / n)
        for lanes, sc in res.items():
            assert np.all(np.abs(sc - ref) <= 4 * sig + 1e-3), (beads, lanes, sc, ref)


def test_rpsh_one_launch_is_bitwise_the_per_bead_count_kernels():
    """One persistent launch serving every bead count runs each trajectory
    with the same lane-group shape as the concurrent per-bead-count kernels,
    and the random stream is keyed by trajectory, so the results are bitwise
    equal whatever order the queues hand trajectories out in."""
    n = 6000
    r0, v0, nb, models = C.rpsh_inputs(n)
    out = {}
    for one in (0, 1):
        eng = C.rpsh_tully(L, n, L.PREC_FP32, max_hops=8)
        try:
            eng.set_mapping(dict(rp_one_launch=one))
            eng.set_initial(np.ascontiguousarray(r0), np.ascontiguousarray(v0), nbeads=np.ascontiguousarray(nb))
            eng.set_trajectory_models(np.ascontiguousarray(models))
            eng.run(0.0, 20000.0, 1.0, 9)
            fin = eng.get_final(32)
            fin["hop_log"] = eng.get_hop_log(8)
            out[one] = fin
        finally:
            eng.close()
    for key in ("r", "v", "state", "nhops", "nsteps", "hop_log"):
        np.testing.assert_array_equal(out[1][key], out[0][key], err_msg=key)


def test_mapping_rejects_unknown_shapes():
    w, c, _, _ = WL.spin_boson_inputs(8, 100)
    eng = C.spinboson_fssh(L, w, c, 8, 100, L.PREC_FP32)
    try:
        for bad in (dict(sb_lanes=3), dict(sb_block=96), dict(rp_lanes={4: 8}), dict(rp_lanes={32: 2}),
                    dict(iesh_cores=2), dict(rp_one_launch=2), dict(iesh_lu_always=2)):
            with pytest.raises(L.EngineError) as e:
                eng.set_mapping(bad)
            assert e.value.code == L.NQCD_ERR_ARG
        with pytest.raises(L.EngineError) as e:  # FP64 accumulators: the 4-lane kernel only
            eng.set_mapping(dict(sb_lanes=8))
        assert e.value.code == L.NQCD_ERR_UNSUPPORTED
    finally:
        eng.close()
