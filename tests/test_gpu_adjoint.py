"""Hand-written adjoint kernels through torch.autograd: gradients of
L = sum_b w_b P_nu(k_b) + 0.5 ||corrected grid||^2 with respect to the grid, the delta_tot
history and the neutrino mass, against the FP64 reference adjoint and against central
finite differences of the FP64 reference step (relative step 1e-6) on 64 grid modes,
64 history entries and the mass.  Stored vs recomputed QAG subdivisions agree."""
import ctypes as C
import math

import numpy as np
import pytest

import adjoint_ref
import cases
import workloads as W

pytestmark = pytest.mark.gpu


def setup(oracle, gpu, N, nb, Na, masses, seed=0):
    c = cases.make_case(N, nb, Na, 1.0 if Na > 64 else 0.5, masses, seed=seed)
    bg, s = cases.oracle_state(oracle, c)
    adjoint_ref.bind(oracle)
    dc0 = np.sqrt(W.spectrum(c["kphys"]))
    P = C.POINTER(C.c_double)
    assert oracle.L.ko_delta_tot_init(s, c["nk"], np.ascontiguousarray(c["kphys"]).ctypes.data_as(P),
                                      dc0.ctypes.data_as(P), c["a_end"]) == 0
    st = oracle.get_state(s)
    vec = (st["nu_init"][:c["nk"]].copy(), st["nu_last"][:c["nk"]].copy(), c["kphys"].copy())
    a = c["a_end"] + 0.01
    ref = adjoint_ref.StepRef(oracle, bg, s, N, nb, c["L"], a, c["count"], c["kphys"], c["scalefact"])
    k = cases.gpu_instance(gpu, c)
    k.set_vectors(*vec)
    return c, ref, k, a


def gpu_grads(k, c, a, wb, recompute, mass_device="cpu"):
    import torch
    from autograd import NeutrinoStep
    step = NeutrinoStep(k, c["scalefact"], a, c["L"], recompute=recompute)
    grid = torch.as_tensor(c["grid"]).cuda().requires_grad_(True)
    hist = torch.as_tensor(c["delta_tot"]).cuda().requires_grad_(True)
    m = torch.tensor(c["MNu"], dtype=torch.float64, device=mass_device, requires_grad=True)
    out, pnu = step(grid, hist, m)
    w = torch.as_tensor(wb).cuda()
    loss = (w * pnu).sum() + 0.5 * torch.view_as_real(out).pow(2).sum()
    loss.backward()
    assert m.grad.device == m.device
    return (grid.grad.detach().cpu().numpy(), hist.grad.detach().cpu().numpy(), m.grad.detach().cpu().numpy(),
            out.detach().cpu().numpy(), pnu.detach().cpu().numpy())


@pytest.mark.parametrize("N,nb,Na", [(64, 48, 24), (256, 128, 128)])
def test_gradients(gpu, oracle, N, nb, Na):
    c, ref, k, a = setup(oracle, gpu, N, nb, Na, (0.05, 0.05, 0.05))
    rng = np.random.default_rng(N)
    wb = rng.random(c["nk"])
    xg, Dg, mg, out, pnu = gpu_grads(k, c, a, wb, recompute=False)
    x = c["grid"].astype(np.complex128)
    D = c["delta_tot"]
    mJ = np.array(c["MNu"])
    adj = ref.adjoint(x, D, mJ, wb)
    f = adj["f"]
    # forward agrees with the reference step (|F|^2 rounded to float as the reference
    # forms it; the rest in FP64)
    f32 = ref.forward(x, D, mJ, wb, f32=True)
    assert cases.rel_err(pnu, f32["out"] ** 2) < 1e-6
    # against the FP64 reference adjoint
    xr = adj["xbar"]
    assert np.max(np.abs(xg - xr)) <= 1e-5 * np.max(np.abs(xr))
    Dr = adj["Dbar"]
    assert np.max(np.abs(Dg - Dr)) <= 1e-5 * np.max(np.abs(Dr))
    assert abs(mg[0] / adj["mbar"][0] - 1) < 1e-5
    # against central finite differences of the FP64 step (64 modes, 64 entries, mass)
    flat = xg.ravel()
    worst = 0.0
    for _ in range(32):
        idx = int(rng.integers(1, x.size))
        for part in (0, 1):
            v = x.ravel()[idx].real if part == 0 else x.ravel()[idx].imag
            if abs(v) < 1e-30:
                continue
            fd = ref.fd_mode(x, D, mJ, wb, f, idx, part)
            got = flat[idx].real if part == 0 else flat[idx].imag
            worst = max(worst, abs(fd - got) / abs(fd))
    assert worst < 1e-5, worst
    errs = []
    for _ in range(64):
        b, j = rng.integers(c["nk"]), rng.integers(D.shape[1])
        errs.append(abs(ref.fd_history(x, D, mJ, wb, f, b, j) - Dg[b, j]))
    assert max(errs) <= 1e-5 * np.max(np.abs(Dg)), max(errs)
    fd = ref.fd_mass(x, D, mJ, wb, f)
    assert abs(fd / mg[0] - 1) < 1e-5, (fd, mg[0])
    # recomputing the subdivisions in the backward pass gives the same gradients
    xg2, Dg2, mg2, _, _ = gpu_grads(k, c, a, wb, recompute=True)
    assert np.array_equal(xg2, xg)
    assert np.max(np.abs(Dg2 - Dg)) <= 1e-14 * np.max(np.abs(Dg))
    assert abs(mg2[0] - mg[0]) <= 1e-14 * abs(mg[0])
    k.close()


def test_mass_gradient_three_mass_states(gpu, oracle):
    """Non-degenerate masses (0.02, 0.03, 0.06 eV: three mass states): the gradient with
    respect to each mass against the FP64 reference adjoint and central differences,
    with the masses on the GPU."""
    c, ref, k, a = setup(oracle, gpu, 64, 48, 24, (0.02, 0.03, 0.06), seed=5)
    wb = np.random.default_rng(7).random(c["nk"])
    xg, Dg, mg, _, _ = gpu_grads(k, c, a, wb, recompute=False, mass_device="cuda")
    x = c["grid"].astype(np.complex128)
    mJ = np.array(c["MNu"])
    adj = ref.adjoint(x, c["delta_tot"], mJ, wb)
    for i in range(3):
        assert abs(mg[i] / adj["mbar"][i] - 1) < 1e-5, (i, mg[i], adj["mbar"][i])
        fd = ref.fd_mass(x, c["delta_tot"], mJ, wb, adj["f"], i=i)
        assert abs(fd / mg[i] - 1) < 1e-5, (i, fd, mg[i])
    k.close()


def test_second_forward_before_backward_is_refused(gpu, oracle):
    """The adjoint reads the state the last forward left in the instance: a backward
    whose forward was followed by another one is refused (KSPACE_ERR_ORDER) rather than
    computed from the second step."""
    import torch
    from autograd import NeutrinoStep
    c, ref, k, a = setup(oracle, gpu, 32, 32, 10, (0.1, 0.1, 0.1))
    step = NeutrinoStep(k, c["scalefact"], a, c["L"])
    grid = torch.as_tensor(c["grid"]).cuda().requires_grad_(True)
    hist = torch.as_tensor(c["delta_tot"]).cuda()
    m = torch.tensor(c["MNu"], dtype=torch.float64)
    out1, p1 = step(grid, hist, m)
    out2, p2 = step(grid, hist * 1.01, m)
    with pytest.raises(gpu.KspaceError) as e:
        out1.abs().pow(2).sum().backward()
    assert e.value.code == 10003
    # the latest forward's backward still works
    out2.abs().pow(2).sum().backward()
    assert torch.isfinite(torch.view_as_real(grid.grad)).all()
    k.close()
