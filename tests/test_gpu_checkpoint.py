"""Checkpoint and resume of device-resident runs (Security_Copy_Cheb /
Restart_State_Cheb, backup.f:329-445): propagate, snapshot, restore into a
fresh trajectory, propagate again -- the populations and Psi equal the
uninterrupted run's bit for bit; the file reads back through the reference's
layout (dynemol_gb300/io.py)."""
import os

import numpy as np
import pytest

from dynemol_gb300 import io, systems

pytestmark = pytest.mark.gpu


def _make(elhl, sysm, coords=None, **kw):
    tr = elhl.Trajectory(sysm, coords=coords, **kw)
    return tr


@pytest.mark.parametrize("case", ["cheb_fp64", "cheb_fp32", "cheb_df64", "taylor"])
def test_fixed_nuclei_resume_is_exact(elhl, flake, tmp_path, case):
    kw = dict(dt=1e-4)
    if case != "taylor":
        prec = {"cheb_fp64": elhl.PREC_FP64, "cheb_fp32": elhl.PREC_FP32, "cheb_df64": elhl.PREC_DF64}[case]
        kw.update(method=elhl.METHOD_CHEBYSHEV, precision=prec, ncols=4, cheb_tol=1e-14)
    path = str(tmp_path / "Security_copy.dat")
    a = _make(elhl, flake, **kw)
    a.init_fmo(41, 40)
    a.step(None, nsteps=3)
    a.snapshot(path)
    pa = a.step(None, nsteps=4)
    ba, ka = a.get_psi()
    sa = a.stats()
    a.close()
    b = _make(elhl, flake, **kw)
    b.init_fmo(41, 40)  # overwritten by the restore
    b.restore(path)
    pb = b.step(None, nsteps=4)
    bb, kb = b.get_psi()
    sb = b.stats()
    b.close()
    assert np.array_equal(pa, pb)
    assert np.array_equal(ka, kb) and np.array_equal(ba, bb)
    assert sa.it == sb.it and sa.t == sb.t
    ck = io.read_checkpoint(path)
    assert ck["it"] == 4 and abs(ck["t"] - 3e-4) < 1e-15
    assert ck["ao_ket"].shape == (flake.nao, 2) and ck["tags"] == ["el", "hl"]
    assert ck["net_charge"].shape == (flake.natoms,)


def test_moving_nuclei_resume_is_exact(elhl, tmp_path):
    sysm = systems.cubic_cluster(n_atoms=64, seed=7)
    coords = np.stack([systems.perturbed_coords(sysm.coords, i, seed=3) for i in range(7)])
    kw = dict(dt=5e-4, method=elhl.METHOD_CHEBYSHEV, precision=elhl.PREC_FP64, ncols=4, cheb_tol=1e-14)
    path = str(tmp_path / "Security_copy.dat")
    a = elhl.Trajectory(sysm, coords=coords[0], **kw)
    a.init_fmo(41, 40)
    a.step(coords[1:3], nsteps=2)
    a.snapshot(path)
    pa = a.step(coords[3:7], nsteps=4)
    a.close()
    b = elhl.Trajectory(sysm, coords=coords[0], **kw)
    b.restore(path)
    pb = b.step(coords[3:7], nsteps=4)
    b.close()
    assert np.array_equal(pa, pb)


def test_server_request_resume(elhl, tmp_path):
    """A request checkpointed after 3 server steps and resubmitted with the
    remaining steps ends with the same populations and Psi as the original."""
    sysm = systems.cubic_cluster(n_atoms=50, seed=21)
    homo = systems.fermi_state(sysm, sysm.fragment_atoms("E"))
    path = str(tmp_path / "req.dat")
    sv = elhl.Server(4e9, dt=1e-4, precision=elhl.PREC_FP32, cheb_tol=1e-12)
    rid = sv.submit(sysm, 8, [homo + 1, homo])
    for _ in range(3):
        sv.step()
    sv.snapshot(rid, path)
    while rid not in sv.poll():
        sv.step()
    p1, k1, _ = sv.result(rid)
    sv.close()
    assert io.read_checkpoint(path)["it"] == 4
    sv = elhl.Server(4e9, dt=1e-4, precision=elhl.PREC_FP32, cheb_tol=1e-12)
    rid = sv.submit(sysm, 5, [homo + 1, homo], restart=path)
    while rid not in sv.poll():
        sv.step()
    p2, k2, _ = sv.result(rid)
    sv.close()
    assert np.array_equal(p1, p2) and np.array_equal(k1, k2)


def test_restore_rejects_a_mismatched_file(elhl, flake, tmp_path):
    path = str(tmp_path / "ck.dat")
    a = elhl.Trajectory(flake, dt=1e-4, method=elhl.METHOD_CHEBYSHEV, precision=elhl.PREC_FP64, ncols=2)
    a.init_fmo(41, 40)
    a.step(None, nsteps=1)
    a.snapshot(path)
    a.close()
    b = elhl.Trajectory(flake, dt=1e-4, method=elhl.METHOD_CHEBYSHEV, precision=elhl.PREC_FP32, ncols=2)
    with pytest.raises(elhl.ElhlError) as e:
        b.restore(path)
    b.close()
    assert e.value.status == elhl.ERR_BAD_ARG
    with open(path, "r+b") as f:  # truncated file
        f.truncate(os.path.getsize(path) // 2)
    c = elhl.Trajectory(flake, dt=1e-4, method=elhl.METHOD_CHEBYSHEV, precision=elhl.PREC_FP64, ncols=2)
    with pytest.raises(elhl.ElhlError):
        c.restore(path)
    c.close()
