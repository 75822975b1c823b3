"""Unrolled gradient-descent reconstruction at the full equal-angle fan
geometry: 512^2 pixels of 0.7 mm, 984 views over 360 degrees, 888 bins of
0.0011 rad, source 541 mm and detector 408 mm from the centre.

Two ellipse phantoms are projected, the noiseless line integrals turned into
Poisson log data (I0 = 1e5, counts clamped >= 1, seed 11), and 10 iterations
x <- x - a A^T(A x - y) from x = 0 (a = 1 / lambda_max(A^T A)) are
backpropagated through ``ctlib_gb300.recon.unrolled_gd`` with per-iteration
checkpointing. The gradient of 0.5 ||x_10 - x_true||^2 with respect to y is
compared with the same recursion run, forward and then in reverse, with

* the FP64 oracle's A and A^T (rel-L2 <= 1e-5), and
* the reference's own kernels prj_fan_ea and prj_t_fan_ea
  (src/fan_ea_kernel.cu:23-472) on this GPU, in fp32 as a reference user gets
  them: the package is within the reference's own distance from the FP64
  recursion, plus 1e-5, of the reference.
"""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

ITERS = 10


@pytest.fixture(scope="module")
def setup(oracle_mod):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import ctlib_gb300 as ct
    from ctlib_gb300 import _native, recon
    from ctlib_gb300.workloads import fan_ea_512, phantoms
    _native.build()
    w = fan_ea_512(2)
    opts = w.slices[0].options
    o32 = torch.tensor(opts, dtype=torch.float32)
    x_true = np.stack(phantoms(w))[:, None]
    xt = torch.from_numpy(x_true).cuda()
    ax = ct.projection(xt, o32).cpu().numpy()
    y_np = recon.poisson_log_sinogram(ax, 1e5, 11)
    step = recon.gd_step_size(o32, 512, 512, torch.device("cuda"))
    return ct, recon, opts, o32, x_true, y_np, step


def _reverse_recursion(A, At, y, x_true, step, iters, zeros):
    """dL/dy of L = 0.5 ||x_K - x_true||^2 for x_{k+1} = x_k - step A^T(A x_k - y)."""
    xs = zeros
    for _ in range(iters):
        xs = xs - step * At(A(xs) - y)
    gx = xs - x_true
    gy = None
    for _ in range(iters):
        t = step * A(gx)
        gy = t if gy is None else gy + t
        gx = gx - step * At(A(gx))
    return gy


def test_unrolled_gd_gradient_full_size(setup, oracle_mod):
    ct, recon, opts, o32, x_true, y_np, step = setup
    O = oracle_mod
    assert 0 < step < 1e-3
    y = torch.from_numpy(y_np).cuda().requires_grad_(True)
    xt = torch.from_numpy(x_true).cuda()
    x = recon.unrolled_gd(y, o32, ITERS, step)
    loss = 0.5 * ((x - xt) ** 2).sum()
    loss.backward()
    got = y.grad.double().cpu().numpy()
    assert np.isfinite(got).all()

    # FP64 oracle recursion on the host
    A = lambda v: O.run("projection", v, opts, O.MODE_F64_ON_F32)
    At = lambda v: O.run("projection_t", v, opts, O.MODE_F64_ON_F32)
    g64 = _reverse_recursion(A, At, y_np.astype(np.float64), x_true.astype(np.float64), step, ITERS,
                             np.zeros_like(x_true, dtype=np.float64))
    e_ours = O.rel_l2(got, g64)
    assert e_ours <= 1e-5, e_ours

    # the reference's kernels on this GPU, fp32
    from oracle import ref_cuda
    if not ref_cuda.available():
        pytest.skip("reference cubins not built")
    ref = ref_cuda.get()
    od = torch.tensor(opts, dtype=torch.float32, device="cuda")
    yr = torch.from_numpy(y_np).cuda()
    gref = _reverse_recursion(lambda v: ref.run(0, v.contiguous(), od), lambda v: ref.run(1, v.contiguous(), od),
                              yr, xt, step, ITERS, torch.zeros_like(xt)).double().cpu().numpy()
    e_ref = O.rel_l2(gref, g64)
    e_ours_ref = O.rel_l2(got, gref)
    print(f"unrolled GD dL/dy: ours vs FP64 {e_ours:.2e}, reference kernels vs FP64 {e_ref:.2e}, "
          f"ours vs reference {e_ours_ref:.2e}")
    assert e_ours_ref <= e_ref + 1e-5, (e_ours_ref, e_ref)


def test_unrolled_gd_checkpoint_matches_plain(setup):
    """Checkpointing changes what is stored, never the values: the gradient with
    and without per-iteration checkpointing is identical."""
    ct, recon, opts, o32, x_true, y_np, step = setup
    xt = torch.from_numpy(x_true).cuda()
    grads = []
    for ckpt in (True, False):
        y = torch.from_numpy(y_np).cuda().requires_grad_(True)
        x = recon.unrolled_gd(y, o32, 3, step, use_checkpoint=ckpt)
        (0.5 * ((x - xt) ** 2).sum()).backward()
        grads.append(y.grad)
    assert torch.equal(grads[0], grads[1])

