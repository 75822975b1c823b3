"""What compensated summation buys, on the precision stress geometry: fan
equal-distance, 1024^2 pixels of 0.33 mm with a fine N(0, 1e-3) texture over
the ellipses, 2304 views, 1472 bins of 0.6429 mm.

For two slices, projection, projection_t (of the phantoms' FP64 sinograms) and
fbp run twice on their own plan: with the default compensated sums
(ctgb_plan_set_summation(plan, 1): plain fp32 blocks folded into a Kahan total)
and with one plain fp32 running sum per output (0), the reference's way of
accumulating (src/fan_ed_kernel.cu:360-401). Both are measured against the FP64
oracle. Compensated must be within 1e-5 and no worse than plain; the default
plan must give the compensated results bit for bit.
"""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def data(oracle_mod):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import ctlib_gb300 as ct
    from ctlib_gb300 import _native
    from ctlib_gb300.ops import Plan
    from ctlib_gb300.workloads import fan_ed_1024, phantoms
    _native.build()
    O = oracle_mod
    w = fan_ed_1024(2)
    opts = w.slices[0].options
    img = np.stack(phantoms(w))[:, None]
    sino = O.run("projection", img, opts, O.MODE_F64_ON_F32).astype(np.float32)
    plan = Plan(tuple(float(v) for v in opts), torch.float32, 0)
    return ct, O, opts, img, sino, plan


_OPS = {"projection": 0, "projection_t": 1, "fbp": 4}


@pytest.mark.parametrize("op", ["projection", "projection_t", "fbp"])
def test_compensated_vs_plain_summation(data, op):
    ct, O, opts, img, sino, plan = data
    x = img if op == "projection" else sino
    xd = torch.from_numpy(x).cuda()
    V, D, W, H = (int(opts[i]) for i in range(4))
    shape = (x.shape[0], 1, V, D) if op == "projection" else (x.shape[0], 1, H, W)
    want = O.run(op, x, opts, O.MODE_F64_ON_F32)
    err = {}
    for comp in (True, False):
        plan.set_summation(comp)
        out = torch.empty(shape, dtype=torch.float32, device="cuda")
        plan.run(_OPS[op], xd, out)
        torch.cuda.synchronize()
        err[comp] = O.rel_l2(out.cpu().numpy(), want)
        if comp:
            default = getattr(ct, op)(xd, torch.tensor(opts, dtype=torch.float32))
            assert torch.equal(out, default)
    plan.set_summation(True)
    print(f"{op}: compensated {err[True]:.2e}, plain fp32 {err[False]:.2e} (rel-L2 vs FP64)")
    assert err[True] <= 1e-5, err
    assert err[True] <= err[False], err
