"""Differentiable candidate refinement: the FP64 reference's analytic
gradient against its own central finite differences (CPU), then the GB300
forward and hand-written adjoint against FP64 central finite differences
(relative error < 1e-3) and the FP64 reference gradient, through a
torch.autograd.Function that wraps the C ABI, and a short Adam fit."""
import numpy as np
import pytest

import synth

NCH, NS, TS = 64, 512, 1.048576e-3
F0, DF = 468.75, -(468.75 - 375.0) / 64


def _case(n=4, seed=11):
    import refine_ref as rr

    g = rr.Geometry(NCH, NS, TS, F0, DF)
    grid = np.arange(0.0, 2001.0, 25.0)
    truth, dm_ref, theta0 = synth.refine_truth(n, grid, nchan=NCH, nsamp=NS, seed=seed)
    rng = np.random.default_rng(seed)
    cut = np.stack([g.model(truth[i], dm_ref[i]) + rng.standard_normal((NCH, NS)) for i in range(n)])
    return g, truth, dm_ref, theta0, cut.astype(np.float32)


def test_reference_gradient_matches_fd():
    g, truth, dm_ref, theta0, cut = _case()
    for i in range(len(cut)):
        th = theta0[i].astype(np.float64)
        an, fd = g.grad(cut[i], th, dm_ref[i]), g.fd_grad(cut[i], th, dm_ref[i])
        assert np.allclose(an, fd, rtol=1e-5, atol=1e-6 * np.abs(fd).max())


# ------------------------------------------------------------------- GPU

def _torch_fn(hella, r):
    import torch

    class Chi2(torch.autograd.Function):
        """chi2(theta) of every cutout through hella_refine_forward, gradient
        through the hand-written adjoint hella_refine_adjoint."""

        @staticmethod
        def forward(ctx, theta, cut, dm_ref):
            out = torch.empty(theta.shape[0], device=theta.device, dtype=torch.float32)
            r.forward(cut, dm_ref, theta.contiguous(), out)
            ctx.save_for_backward(theta, cut, dm_ref)
            return out

        @staticmethod
        def backward(ctx, g):
            theta, cut, dm_ref = ctx.saved_tensors
            gt = torch.empty_like(theta)
            r.adjoint(cut, dm_ref, theta.contiguous(), g.contiguous(), gt)
            return gt, None, None

    return Chi2.apply


@pytest.mark.gpu
def test_gpu_forward_and_adjoint_vs_fp64(hella):
    import torch

    g, truth, dm_ref, theta0, cut = _case(n=6, seed=12)
    r = hella.Refine(8, NCH, NS, TS, F0, DF, stream=torch.cuda.current_stream().cuda_stream)
    assert np.array_equal(r.delay_table(), g.tab.astype(np.float32))
    chi2 = _torch_fn(hella, r)
    dcut = torch.from_numpy(cut).cuda()
    ddm = torch.from_numpy(dm_ref).cuda()
    theta = torch.from_numpy(theta0).cuda().requires_grad_(True)
    loss = chi2(theta, dcut, ddm)
    loss.sum().backward()
    got_chi2 = loss.detach().cpu().numpy()
    got_grad = theta.grad.cpu().numpy()
    for i in range(len(cut)):
        th = theta0[i].astype(np.float64)
        want = g.chi2(cut[i], th, dm_ref[i])
        assert abs(got_chi2[i] - want) <= 1e-4 * want
        fd = g.fd_grad(cut[i], th, dm_ref[i])
        an = g.grad(cut[i], th, dm_ref[i])
        for k in range(5):
            assert abs(got_grad[i, k] - fd[k]) <= 1e-3 * abs(fd[k]) + 1e-6 * np.abs(fd).max(), (i, k, got_grad[i], fd)
            assert abs(got_grad[i, k] - an[k]) <= 1e-3 * abs(an[k]) + 1e-6 * np.abs(an).max()


@pytest.mark.gpu
def test_gpu_adam_fit_improves_dm(hella):
    import torch

    g, truth, dm_ref, theta0, cut = _case(n=16, seed=13)
    r = hella.Refine(16, NCH, NS, TS, F0, DF, stream=torch.cuda.current_stream().cuda_stream)
    dcut = torch.from_numpy(cut).cuda()
    ddm = torch.from_numpy(dm_ref).cuda()
    theta = torch.from_numpy(theta0).cuda()
    c0 = torch.empty(16, device="cuda")
    r.forward(dcut, ddm, theta, c0)
    c1 = torch.empty(16, device="cuda")
    r.fit(dcut, ddm, theta, 200, [0.5, 0.2, 0.05, 0.05, 0.05], c1)
    torch.cuda.synchronize()
    fit = theta.cpu().numpy()
    assert np.all(c1.cpu().numpy() <= c0.cpu().numpy() * 1.0001)
    err0 = np.abs(theta0[:, 0] - truth[:, 0])
    err1 = np.abs(fit[:, 0] - truth[:, 0])
    assert np.median(err1) < np.median(err0)
