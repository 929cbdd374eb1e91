"""GPU test of the allocation-free entry point elhl_propagate_fixed_scratch.

It is meant for callers that cannot allocate device memory (a pool allocator
owns the device, a graph capture is in progress elsewhere, or allocation's
implicit synchronisation is not acceptable).  The test calls it through the C
ABI on device buffers and checks it against the existing
propagation_gpucaller_ entry point on the same inputs, for three calls in a
row.  Each continues from the last, so it also sees the array's leftover
contents from the previous call.  The second call runs on a non-default
stream, and the third checks that the device's free memory does not change.
This file sorts last so that a stop-at-first-
failure run has already run every other test."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_fixed_scratch_matches_gpucaller(elhl, oracle_mod, flake):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    S = oracle_mod.overlap(flake)
    h = oracle_mod.huckel(flake, S)
    Hp = oracle_mod.h_prime(oracle_mod.sy_invert(S), h)
    bra, ket = oracle_mod.initial_states(flake, S, 41, 40)
    N = flake.nao
    ld = N + 6  # a leading dimension larger than n
    Hpad = np.zeros((ld, N), order="F")
    Hpad[:N, :] = Hp
    d_H = torch.from_numpy(np.asfortranarray(Hpad).T.copy()).to(dev)  # column j contiguous, stride ld
    ref_b = np.ascontiguousarray(bra[:, 0])
    ref_k = np.ascontiguousarray(ket[:, 0])
    d_b = torch.from_numpy(ref_b.view(np.float64).copy()).to(dev)
    d_k = torch.from_numpy(ref_k.view(np.float64).copy()).to(dev)
    tau_max = 1e-4 / oracle_mod.H_BAR
    side = torch.cuda.Stream(dev)
    t = 0.0
    for call in range(3):
        t_max = t + 1e-4
        ref_b, ref_k, ref_st = elhl.propagation_gpucaller(Hp, ref_b, ref_k, t, t_max, tau_max)
        # call 1 runs on a stream of its own; calls 0 and 2 on torch's current stream
        stream = side if call == 1 else torch.cuda.current_stream(dev)
        stream.wait_stream(torch.cuda.current_stream(dev))
        torch.cuda.synchronize(dev)
        free_before = torch.cuda.mem_get_info(dev)[0]
        st = elhl.propagate_fixed_scratch(N, d_H.data_ptr(), ld, d_b.data_ptr(), d_k.data_ptr(), t, t_max, tau_max,
                                          stream.cuda_stream)
        free_after = torch.cuda.mem_get_info(dev)[0]
        if call == 2:
            # the module and its array are resident after the first calls: no device memory is taken
            assert free_after == free_before
        got_b = d_b.cpu().numpy().view(np.complex128)
        got_k = d_k.cpu().numpy().view(np.complex128)
        assert st == pytest.approx(ref_st, rel=1e-12)
        assert np.abs(got_k - ref_k).max() < 1e-12
        assert np.abs(got_b - ref_b).max() < 1e-12
        t = t_max


def test_fixed_scratch_rejects_oversize(elhl):
    with pytest.raises(elhl.ElhlError) as e:
        elhl.propagate_fixed_scratch(elhl.FIXED_SCRATCH_MAX_N + 1, 1, elhl.FIXED_SCRATCH_MAX_N + 1, 1, 1, 0.0, 1e-4, 0.1)
    assert e.value.status == elhl.ERR_BAD_ARG
