"""FileReduction of the host mirror (nqcd_gb300.api) against the layout of
the reference's FileReduction (src/Ensembles/reductions.jl:57-91): one group
`trajectory_<id>` per trajectory, ids from 1, one dataset per output key plus
`Time`; numbers and arrays written as they are, vectors of arrays stacked on a
trailing axis; outputs of other types refused.  The container is .npz (no HDF5
library here), with the group/dataset path as the array name."""
import numpy as np
import pytest

import nqcd_gb300 as N
from nqcd_gb300 import api


def fake_final(n, ndof):
    rng = np.random.default_rng(3)
    return dict(r=rng.normal(size=(n, ndof)), v=rng.normal(size=(n, ndof)), energy=rng.normal(size=(n, 2)),
                nhops=rng.integers(0, 5, n).astype(np.int32))


def test_filename_takes_the_npz_extension():
    assert N.FileReduction("out.h5").filename == "out.npz"
    assert N.FileReduction("dir/out.hdf5").filename == "dir/out.npz"
    assert N.FileReduction("out").filename == "out.npz"
    assert N.FileReduction("out.npz").filename == "out.npz"


def test_groups_per_trajectory(tmp_path):
    n, ndof = 5, 3
    fin = fake_final(n, ndof)
    r0, v0 = np.ones((n, ndof)), -np.ones((n, ndof))
    outputs = (N.OutputTotalEnergy, N.OutputSurfaceHops, N.OutputPosition, N.OutputVelocity)
    red = N.FileReduction(str(tmp_path / "ens.h5"))
    msg = red.write([0.0, 2.5], api._per_trajectory(outputs, fin, (r0, v0), hops=True))
    assert msg == f"Output written to {tmp_path / 'ens.npz'}."
    f = np.load(tmp_path / "ens.npz")
    assert sorted(f.files) == sorted(f"trajectory_{i}/{k}" for i in range(1, n + 1)
                                     for k in ("Time", "OutputTotalEnergy", "OutputSurfaceHops", "OutputPosition",
                                               "OutputVelocity"))
    for i in range(n):
        g = f"trajectory_{i + 1}/"
        np.testing.assert_array_equal(f[g + "Time"], [0.0, 2.5])
        np.testing.assert_array_equal(f[g + "OutputTotalEnergy"], fin["energy"][i])
        assert f[g + "OutputSurfaceHops"] == fin["nhops"][i]
        # vector of (ndof,) arrays stacked on the trailing axis: (ndof, 2)
        np.testing.assert_array_equal(f[g + "OutputPosition"], np.stack([r0[i], fin["r"][i]], axis=-1))
        np.testing.assert_array_equal(f[g + "OutputVelocity"], np.stack([v0[i], fin["v"][i]], axis=-1))


def test_ring_polymer_positions_keep_the_bead_axis(tmp_path):
    n, nb = 4, 3
    fin = fake_final(n, nb)
    r0 = np.arange(n * nb, dtype=float).reshape(n, nb)
    red = N.FileReduction(str(tmp_path / "rp.npz"))
    red.write([0.0, 1.0], api._per_trajectory((N.OutputPosition,), fin, (r0, r0), hops=False))
    f = np.load(tmp_path / "rp.npz")
    assert f["trajectory_2/OutputPosition"].shape == (nb, 2)
    np.testing.assert_array_equal(f["trajectory_2/OutputPosition"][:, 0], r0[1])


def test_outputs_that_are_not_arrays_are_refused():
    fin = fake_final(2, 1)
    with pytest.raises(TypeError, match="Cannot convert"):
        api._per_trajectory((N.OutputFinal,), fin, None, hops=True)
    with pytest.raises(TypeError, match="Cannot convert"):
        api._per_trajectory((N.OutputSurfaceHops,), fin, None, hops=False)  # MDEF has no hops
    with pytest.raises(TypeError, match="Cannot convert"):
        api._per_trajectory((N.OutputPosition,), fin, None, hops=True)  # initial conditions drawn on the device


def test_other_reductions_are_refused_before_any_engine():
    with pytest.raises(NotImplementedError):
        N.run_dynamics(None, (0.0, 1.0), N.DynamicalDistribution(np.zeros(1), np.zeros(1), (1, 1)) * N.PureState(1),
                       output=N.OutputTotalEnergy, reduction=api.SortByTrajectoryReduction())
