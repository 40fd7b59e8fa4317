"""applyMPO, compressTwoSite, compress and compressSingleSite on the GPU against the oracle's
restatements: the same block structure and values for W|psi>, the same convergence measures and the
same fitted states (dense amplitudes) for binding and non-binding bond dimensions."""
import numpy as np
import pytest

import ed
from mpstools_gb300 import api, models as M
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu


def _case(N=8, chi=8, seed=3):
    Jz = M.xxz_couplings(N, 1)
    W = M.heisenberg_mpo(Jz, np.ones(N - 1), np.zeros(N))
    return W, M.u1_itokeys(N), M.random_u1_mps(N, N // 2, chi, seed)


def test_apply_mpo_matches_oracle(ctx):
    W, ik, psi = _case()
    got = api.applyMPO(W, psi, ik, ctx=ctx)
    ref = O.apply_mpo(psi, W, ik)
    for g, r in zip(got, ref):
        assert set(g) == set(r)
        for k in r:
            assert g[k].shape == r[k].shape
            assert np.abs(g[k] - r[k]).max() <= 1e-13 * max(1.0, np.abs(r[k]).max())


@pytest.mark.parametrize("chimax", [12, 200])
def test_compress_matches_oracle(ctx, chimax):
    W, ik, psi = _case()
    N = len(psi)
    conv_g, fit_g = api.compressTwoSite(psi, W, ik, chimax=chimax, maxstep=3, delta=1e-12, doTrunc=True,
                                        tr_weight=1e-12, ctx=ctx)
    conv_r, fit_r = O.compress_two_site(psi, W, ik, chimax=chimax, maxstep=3, delta=1e-12, doTrunc=True,
                                        tr_weight=1e-12)
    vg, vr = ed.mps_sector_vector(fit_g, N // 2), ed.mps_sector_vector(fit_r, N // 2)
    print(f"chimax {chimax}: conv gpu {conv_g:.12e} oracle {conv_r:.12e}, "
          f"max amplitude diff {np.abs(vg - vr).max() / np.abs(vr).max():.2e}")
    assert abs(conv_g - conv_r) <= 1e-9 * max(1.0, abs(conv_r))
    assert np.abs(vg - vr).max() <= 1e-9 * np.abs(vr).max()


@pytest.mark.parametrize("chimax,normalize", [(4, False), (200, False), (6, True)])
def test_single_site_compress_matches_oracle(ctx, chimax, normalize):
    W, ik, psi = _case(chi=16)
    N = len(psi)
    conv_g, fit_g = api.compress(psi, ik, chimax=chimax, maxstep=3, delta=1e-14, normalize=normalize, ctx=ctx)
    conv_r, _, fit_r = O.compress(psi, ik, chimax=chimax, maxstep=3, delta=1e-14, normalize=normalize)
    vg, vr = ed.mps_sector_vector(fit_g, N // 2), ed.mps_sector_vector(fit_r, N // 2)
    if normalize:  # the sign of the dropped norm is the boundary SVD's choice
        vg = vg * np.sign(vg @ vr)
    print(f"compress chimax {chimax} normalize {normalize}: conv gpu {conv_g:.12e} oracle {conv_r:.12e}, "
          f"max amplitude diff {np.abs(vg - vr).max() / np.abs(vr).max():.2e}")
    assert abs(conv_g - conv_r) <= 1e-9 * max(1e-3, abs(conv_r))
    assert np.abs(vg - vr).max() <= 1e-9 * np.abs(vr).max()


@pytest.mark.parametrize("chimax", [15, 200])
def test_compress_single_site_matches_oracle(ctx, chimax):
    W, ik, psi = _case(chi=16)
    N = len(psi)
    conv_g, fit_g = api.compressSingleSite(psi, W, ik, chimax=chimax, maxstep=3, delta=1e-14, ctx=ctx)
    conv_r, fit_r = O.compress_single_site(psi, W, ik, chimax=chimax, maxstep=3, delta=1e-14)
    vg, vr = ed.mps_sector_vector(fit_g, N // 2), ed.mps_sector_vector(fit_r, N // 2)
    target = ed.mps_sector_vector(O.apply_mpo(psi, W, ik), N // 2)
    dg, dr = (np.linalg.norm(v - target) / np.linalg.norm(target) for v in (vg, vr))
    print(f"compressSingleSite chimax {chimax}: conv gpu {conv_g:.12e} oracle {conv_r:.12e}, "
          f"max amplitude diff {np.abs(vg - vr).max() / np.abs(vr).max():.2e}, distance to W psi {dg:.4e} / {dr:.4e}")
    if chimax >= 5 * 16:
        # psi is not truncated: the initial guess W psi is the fit, unique
        assert abs(conv_g - conv_r) <= 1e-9 * max(1.0, abs(conv_r))
        assert np.abs(vg - vr).max() <= 1e-9 * np.abs(vr).max()
    else:
        # binding: the initial guess W psi_trunc carries Schmidt values at rounding level (~1e-16)
        # whose vectors are whatever the SVD routine returns, and prepareSite keeps every value above
        # 1e-16, so how many of them survive, and which directions they span, depends on the rounding
        # of the bidiagonalisation; the single-site fit keeps them in its basis, so the fit is not
        # unique: the oracle itself moves by 3e-3 in amplitudes and 1.3e-5 in the measure between two
        # LAPACK SVD drivers.  The GPU fit is a fit of the same kind: the same measure to 1e-3 and a
        # distance to W psi of the same order as the oracle's.
        assert abs(conv_g - conv_r) <= 1e-3 * abs(conv_r)
        assert dg <= 2.5 * dr and dg < 5e-2
