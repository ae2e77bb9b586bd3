"""Differentiable NUFFT: loss ||E(x,k) - y||^2 and its gradients with respect to the
image and the trajectory, against the FP64 oracle and FP64 central finite
differences (step 1e-4 grid units)."""
import numpy as np
import pytest

from tests.helpers import case, rel

pytestmark = pytest.mark.gpu


def _setup(mrg_lib, N, C, nproj, jitter, analytic, seed=31):
    import torch
    c = case(N=N, C=C, nproj=nproj, jitter=jitter, seed=seed)
    c["kw"] = np.ones_like(c["kw"])
    rng = np.random.default_rng(seed)
    M = c["kx"].size
    c["y"] = (0.05 * (rng.standard_normal((C, M)) + 1j * rng.standard_normal((C, M)))).astype(np.complex64)
    p = mrg_lib.Plan(N, C, 1, analytic_kernel=analytic)
    p.set_traj(0, c["kx"], c["ky"], c["kz"], c["kw"])
    p.set_smaps(torch.from_numpy(c["smaps"]).cuda())
    loss, gx, gk = p.grad(0, torch.from_numpy(c["X"]).cuda(), torch.from_numpy(c["y"]).cuda())
    return c, p, loss, gx.cpu().numpy(), gk.cpu().numpy()


def _oracle_loss_gradx(oracle_lib, c, analytic):
    O = oracle_lib.Plan(c["N"], prec=1, k_rad=1e30, analytic=analytic)
    a = (c["kx"], c["ky"], c["kz"], c["kw"])
    loss, gx = 0.0, np.zeros(O.ishape, np.complex128)
    for k in range(c["C"]):
        r = O.forward(c["X"], c["smaps"][k], *a) - c["y"][k]
        loss += float(np.sum(np.abs(r) ** 2))
        gx = O.adjoint(gx, c["smaps"][k], (2 * r).astype(np.complex128), *a)
    return loss, gx


def _fd_gradk(oracle_lib, c, analytic, idx, h_grid=1e-4):
    """Central differences of the loss in each coordinate of the samples idx."""
    O = oracle_lib.Plan(c["N"], prec=1, k_rad=1e30, analytic=analytic)
    g = O.grid_ratio[0]
    h = h_grid / g
    k = [c[n][idx].astype(np.float64) for n in ("kx", "ky", "kz")]
    n = idx.size
    pos = [np.concatenate([k[a] + (h if (d == a and s > 0) else -h if (d == a) else 0.0)
                           for d in range(3) for s in (+1, -1)]) for a in range(3)]
    out = np.zeros((3, n))
    for coil in range(c["C"]):
        v = O.values_at(c["X"], c["smaps"][coil], *pos).reshape(3, 2, n)
        y = c["y"][coil][idx]
        out += (np.abs(v[:, 0] - y) ** 2 - np.abs(v[:, 1] - y) ** 2) / (2 * h)
    return out


def _smooth(c, h_grid=1e-4):
    """Samples whose tap range does not change within +-2h (the kernel is cut at dwin)."""
    S = 16 * int(np.ceil(1.5 * c["N"] / 16))
    g = S / c["N"]
    ok = np.ones(c["kx"].size, bool)
    for n in ("kx", "ky", "kz"):
        dk = c[n].astype(np.float64) * np.float32(g) + S // 2
        for e in (dk - 2.5, dk + 2.5):
            ok &= np.abs(e - np.round(e)) > 4 * h_grid
    return ok


@pytest.mark.parametrize("analytic", [True, False])
def test_loss_and_image_gradient(mrg_lib, oracle_lib, analytic):
    c, p, loss, gx, gk = _setup(mrg_lib, 32, 3, 400, 0.05, analytic)
    lref, gref = _oracle_loss_gradx(oracle_lib, c, analytic)
    assert abs(loss - lref) / lref < 1e-5
    assert rel(gx, gref) < 1e-5


def test_trajectory_gradient_vs_finite_differences(mrg_lib, oracle_lib):
    c, p, loss, gx, gk = _setup(mrg_lib, 32, 3, 400, 0.05, True)
    idx = np.nonzero(_smooth(c))[0]
    idx = idx[::7]
    fd = _fd_gradk(oracle_lib, c, True, idx)
    err = rel(gk[:, idx], fd)
    print("analytic-kernel trajectory gradient vs FP64 central differences: rel-L2 %.3g over %d samples" % (err, idx.size))
    assert err < 1e-4


def test_table_forward_gradient_deviation(mrg_lib, oracle_lib):
    """With the reference's table forward the analytic derivative differs from the
    table's piecewise-linear slope at the table resolution (1/600 grid unit)."""
    c, p, loss, gx, gk = _setup(mrg_lib, 32, 3, 400, 0.05, False)
    idx = np.nonzero(_smooth(c))[0][::7]
    fd_table = _fd_gradk(oracle_lib, c, False, idx)
    fd_analytic = _fd_gradk(oracle_lib, c, True, idx)
    dev = rel(gk[:, idx], fd_table)
    print("table-forward: analytic gradient vs table finite differences %.3g, vs analytic %.3g" %
          (dev, rel(gk[:, idx], fd_analytic)))
    assert dev < 5e-2


def test_torch_autograd_wrapper(mrg_lib):
    import torch
    from mri_recon_gb300.gridfft import NufftLoss
    c, p, loss, gx, gk = _setup(mrg_lib, 32, 3, 300, 0.05, True)
    x = torch.from_numpy(c["X"]).cuda().requires_grad_(True)
    k = torch.from_numpy(np.stack([c["kx"], c["ky"], c["kz"]])).cuda().requires_grad_(True)
    y = torch.from_numpy(c["y"]).cuda()
    L = NufftLoss.apply(x, k, y, p)
    L.backward()
    assert abs(float(L) - loss) / loss < 1e-6
    assert rel(x.grad.cpu().numpy(), gx) < 1e-6
    assert rel(k.grad.cpu().numpy(), gk) < 1e-6
    with torch.no_grad():
        x2 = x - 1e-3 * x.grad / x.grad.abs().max()
    assert float(NufftLoss.apply(x2, k.detach(), y, p)) < float(L)


def test_grad96_configuration(mrg_lib, oracle_lib):
    """96^3, 8 coils, 6000 x 96 radial with 0.05 grid-unit jitter: one instance of the
    batch-of-4 configuration, image gradient against the oracle, trajectory gradient
    against finite differences on a subset of samples."""
    c, p, loss, gx, gk = _setup(mrg_lib, 96, 8, 6000, 0.05, True, seed=1238)
    lref, gref = _oracle_loss_gradx(oracle_lib, c, True)
    assert abs(loss - lref) / lref < 1e-5
    assert rel(gx, gref) < 1e-5
    idx = np.nonzero(_smooth(c))[0][::1500]
    fd = _fd_gradk(oracle_lib, c, True, idx)
    assert rel(gk[:, idx], fd) < 1e-4
