"""Device kinematics (fjg_kinematics) vs the host build of the same integer
code, and vs CUDA's own FP64 log/atan2 (needs a GB300)."""
import numpy as np
import pytest

import oracle
from fastjet_gpu_gb300 import events as E

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import fastjet_gpu_gb300 as F
    return F.Context(0)


def _particles():
    b = E.mixed_batch(64, 50, 2000, seed=5)
    extra = np.array([[0.0, 0.0, 5.0, 5.0], [1.0, 0.0, 0.0, 1.0], [0.0, 1.0, 0.0, 1.0], [-1.0, 0.0, 3.0, 4.0],
                      [0.8064370155, -0.0000000594, 61.86539841, 61.87065887], [1e-9, 1.0, -2.0, 3.0],
                      [3.0, 4.0, 0.0, 5.0], [-3.0, -4.0, 100.0, 101.0]])
    return np.concatenate([b.particles, extra])


def test_device_matches_host_integer_kinematics(ctx):
    import torch
    p = _particles()
    t = torch.from_numpy(p).cuda()
    for algo in (1, 0, -1):
        rap, phi, w = (x.cpu().numpy() for x in ctx.kinematics(t, algo))
        host = np.array([oracle.kin_kinematics(q, algo) for q in p])
        assert np.array_equal(rap, host[:, 0]) and np.array_equal(phi, host[:, 1]) and np.array_equal(w, host[:, 2])


def test_device_agrees_with_cuda_libm(ctx):
    """rapidity and azimuth against CUDA's FP64 log/atan2 on the same inputs.

    Measured on GB300: rapidity identical for 99.94% of the particles (max 1
    ulp); azimuth identical for 93.5% (max 2 ulp) -- CUDA's atan2 is not
    correctly rounded (documented error bound 2 ulp), while fjg_kin.h agrees
    with the correctly rounded value (tests/test_kinematics.py).  The
    clustering decisions do not depend on these last-place differences except
    at exact near-ties: the reference goldens, produced with CUDA's libm,
    are reproduced bit for bit."""
    import torch
    p = _particles()
    t = torch.from_numpy(p).cuda()
    rap, phi, _ = (x.cpu().numpy() for x in ctx.kinematics(t, 1))
    px, py, pz, E_ = p.T
    pt2 = px * px + py * py
    m2 = np.maximum(0.0, (E_ + pz) * (E_ - pz) - pt2)
    epz = E_ + np.abs(pz)
    x = (pt2 + m2) / (epz * epz)
    special = (E_ == np.abs(pz)) & (pt2 == 0)
    lg = torch.log(torch.from_numpy(np.where(special, 1.0, x)).cuda()).cpu().numpy()
    rap_cuda = 0.5 * lg
    rap_cuda = np.where(pz > 0, -rap_cuda, rap_cuda)
    at = torch.atan2(torch.from_numpy(py).cuda(), torch.from_numpy(px).cuda()).cpu().numpy()
    at = np.where(pt2 == 0, 0.0, at)
    phi_cuda = np.where(at < 0, at + 2 * np.pi, at)
    ok = ~special
    r_same = (rap[ok] == rap_cuda[ok]).mean()
    p_same = (phi == phi_cuda).mean()
    ulp_r = np.abs(rap[ok].view(np.int64) - rap_cuda[ok].view(np.int64)).max()
    ulp_p = np.abs(phi.view(np.int64) - phi_cuda.view(np.int64)).max()
    print(f"identical to CUDA libm: rap {r_same:.6f}, phi {p_same:.6f}; max ulp {ulp_r}, {ulp_p}")
    assert ulp_r <= 1 and ulp_p <= 2
    assert r_same >= 0.999 and p_same >= 0.9
