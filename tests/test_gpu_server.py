"""GPU tests of the continuous-batching server: requests that arrive while
others run are admitted at step boundaries within the HBM budget, and each
result is the same alone and in the mix (FP64: 1e-12, FP32: 1e-6)."""
import numpy as np
import pytest

from dynemol_gb300 import systems

pytestmark = pytest.mark.gpu


def _requests():
    out = []
    for i, (n, steps, cols) in enumerate([(30, 3, 2), (64, 5, 4), (20, 2, 2), (48, 4, 6), (36, 6, 2)]):
        sysm = systems.cubic_cluster(n_atoms=n, seed=20 + i)
        homo = systems.fermi_state(sysm, sysm.fragment_atoms("E"))
        states = [homo - c // 2 if c % 2 else homo + 1 + c // 2 for c in range(cols)]
        out.append((sysm, steps, states))
    return out


def _alone(elhl, sysm, steps, states, prec):
    tr = elhl.Trajectory(sysm, dt=1e-4, method=elhl.METHOD_CHEBYSHEV, precision=prec, ncols=len(states),
                         nparticles=len(states), cheb_tol=1e-14)
    tr.init_fmo_states(states)
    pops = tr.step(None, nsteps=steps)
    b, k = tr.get_psi()
    tr.close()
    return pops[-1], k


@pytest.mark.parametrize("prec,tol", [(0, 1e-12), (1, 1e-6)])
def test_server_mix_equals_alone(elhl, prec, tol):
    reqs = _requests()
    # budget for about two of the requests at a time: forces queueing
    sv = elhl.Server(4.5e6, dt=1e-4, precision=prec, cheb_tol=1e-14)
    ids = {}
    ids[sv.submit(*reqs[0])] = 0
    ids[sv.submit(*reqs[1])] = 1
    sv.step()
    for q in range(2, len(reqs)):          # later arrivals join while others run
        ids[sv.submit(*reqs[q])] = q
        sv.step()
    done = {}
    for _ in range(200):
        for rid in sv.poll():
            done[rid] = sv.result(rid)
        if len(done) == len(reqs):
            break
        sv.step()
    assert len(done) == len(reqs)
    for rid, (pops, psi, times) in done.items():
        sysm, steps, states = reqs[ids[rid]]
        ap, ak = _alone(elhl, sysm, steps, states, prec)
        assert np.abs(pops - ap).max() < tol
        assert np.abs(psi - ak).max() < 10 * tol
        assert times[0] <= times[1] <= times[2]
    sv.close()


def test_server_rejects_oversize(elhl):
    sysm = systems.cubic_cluster(n_atoms=64, seed=1)
    sv = elhl.Server(1e5, dt=1e-4)
    with pytest.raises(elhl.ElhlError) as e:
        sv.submit(sysm, 2, [40, 41])
    assert e.value.status == elhl.ERR_OOM
    sv.close()
