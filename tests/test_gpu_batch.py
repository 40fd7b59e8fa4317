"""Batched chains on the GPU: independent XXZ chains of different lengths and couplings swept in
lockstep through one direct-sum problem per step, against the same chains run one by one with the
single-chain engine (DMRGengine::simulate): the same step sequence, kept bond dimensions and
energies (1e-10 relative), and the same energy of the final state.  At any global step the chains
are at different sites and sweep directions."""
import numpy as np
import pytest

from mpstools_gb300 import api, models as M

pytestmark = pytest.mark.gpu


def _chains(lengths, chi, seed0):
    out = []
    for i, N in enumerate(lengths):
        W = M.heisenberg_mpo(M.xxz_couplings(N, 10 + i), np.ones(N - 1), np.zeros(N))
        out.append((M.random_u1_mps(N, N // 2, chi, seed0 + i), W, M.u1_itokeys(N)))
    return out


def _reference(ctx, chains, sweeps, chi, delta, prec="fp64"):
    ref = []
    for sites, W, ik in chains:
        e = api.DMRGengine(sites, W, ik, prec=prec, ctx=ctx)
        E = e.simulate(maxsteps=sweeps, EnConv=1e-300, chimax=chi, doTrunc=False, delta=delta)
        ref.append((E, e.steps(), e.measure_energy()))
        e.close()
    return ref


@pytest.mark.parametrize("prec", ["fp64", "auto", "mixed", "tf32x3"])
def test_batch_matches_independent_chains(ctx, prec):
    lengths, chi, sweeps, delta = [8, 11, 14, 10, 9], 16, 2, 1e-12
    chains = _chains(lengths, chi, 100)
    ref = _reference(ctx, chains, sweeps, chi, delta, prec)
    engines = [api.DMRGengine(s, W, ik, ctx=ctx) for s, W, ik in chains]
    batch = api.DMRGbatch(engines, prec=prec)
    E = batch.simulate(sweeps, chi, doTrunc=False, delta=delta)
    st = batch.stats()
    worst = 0.0
    for i, e in enumerate(engines):
        E_ref, steps_ref, meas_ref = ref[i]
        steps = e.steps()
        assert [(s["site"], s["dir"]) for s in steps] == [(s["site"], s["dir"]) for s in steps_ref]
        assert [s["chi"] for s in steps] == [s["chi"] for s in steps_ref]
        for a, b in zip(steps, steps_ref):
            worst = max(worst, abs(a["E"] - b["E"]) / abs(b["E"]))
        # TF32X3 reports its Ritz values (the batched and the single-chain reductions differ in order)
        assert abs(E[i] - E_ref) <= (1e-6 if prec == "tf32x3" else 1e-10) * abs(E_ref)
        assert abs(e.measure_energy() - meas_ref) <= 1e-10 * abs(meas_ref)
    print(f"{prec}: {len(engines)} chains, worst per-step relative energy difference {worst:.2e}, stats {st}")
    # FP64: the batched and the single-chain Lanczos differ only in the order of their reductions.
    # The tensor-core modes stop their TF32X3 phase on the precision floor, where the order of the
    # reductions decides the stopping iteration: early steps from the random start, before the states
    # converge, land up to a few 1e-8 apart (MIXED; AUTO's FP64 finish brings it to 1e-9; TF32X3's own
    # Ritz values carry the ~5e-6 scaling of FP32 accumulation in both runs); the final energies above
    # agree to 1e-10.
    assert worst <= {"fp64": 1e-12, "auto": 1e-9, "mixed": 1e-7, "tf32x3": 1e-6}[prec]
    # one lockstep step per step of the longest chain; every chain step was done
    assert st["global_steps"] == max(len(r[1]) for r in ref)
    assert st["chain_steps"] == sum(len(r[1]) for r in ref)
    batch.close()
    for e in engines:
        e.close()


@pytest.mark.parametrize("prec", ["mixed", "tf32x3"])
def test_batch_mixed_modes_against_the_oracle(ctx, prec):
    """The tensor-core batched modes against the oracle's FP64 DMRG of each chain: MIXED's final
    energies (FP64 Rayleigh quotients) to 1e-10; TF32X3's final energies are its own Ritz values, off
    by the tensor cores' FP32-accumulation scaling (~5e-6 relative at most on these sizes)."""
    from oracle import pyoracle as O
    lengths, chi, sweeps, delta = [10, 12, 9], 16, 3, 1e-12
    chains = _chains(lengths, chi, 200)
    E_or = [O.DMRG(s, W, ik, maxthreads=4).simulate(maxsteps=sweeps, EnConv=1e-300, chimax=chi, delta=delta)
            for s, W, ik in chains]
    engines = [api.DMRGengine(s, W, ik, ctx=ctx) for s, W, ik in chains]
    batch = api.DMRGbatch(engines, prec=prec)
    E = batch.simulate(sweeps, chi, doTrunc=False, delta=delta)
    batch.close()
    for e in engines:
        e.close()
    tol = 1e-10 if prec == "mixed" else 1e-5
    for a, b in zip(E, E_or):
        assert abs(a - b) <= tol * abs(b), (prec, a, b)
