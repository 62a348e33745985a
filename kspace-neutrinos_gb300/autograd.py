"""torch.autograd wrapper of one neutrino-correction step (hand-written adjoint kernels).

    step = NeutrinoStep(instance, scalefact, Time, BoxSize)
    out, pnu = step(grid, history, masses)      # grid c64 [N,N,N/2+1] (cuda), history f64 [nk, Na] (cuda),
                                                # masses f64 [3] (mass inside J per mass state, eV)
    loss = (w * pnu).sum() + 0.5 * out.abs().pow(2).sum()
    loss.backward()                             # grid.grad, history.grad, masses.grad

The step is add_nu_power_to_rhogrid (interface_gadget.c:158-194) with the integrator
state (delta_nu_init, delta_nu_last, set by KspaceNeutrinos.set_vectors) held fixed and
the history table an input.  Gradients hold every QAG subdivision fixed and the
background Omega_nu(a), H(a) fixed; the mass gradient is through the free-streaming
argument of J.  recompute=True re-runs the integrals in the backward pass instead of
keeping the subdivisions (the memory-light variant).

One forward per backward on an instance: the adjoint reads state the forward leaves in
the instance, so a second forward on the same instance before the first one's backward
makes that backward raise KspaceError (code 10003, KSPACE_ERR_ORDER) instead of
returning the second step's gradients.  Use one instance per step held for backward.
"""
import numpy as np
import torch


class _Fn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, grid, history, masses, inst, scalefact, Time, BoxSize, recompute):
        N = grid.shape[1]
        inst.set_nu_state(scalefact, history.detach().contiguous())
        inst.set_jmass(masses.detach().cpu().numpy())
        out = torch.empty_like(grid)
        nk = history.shape[0]
        pnu = torch.empty(nk, dtype=torch.float64, device=grid.device)
        torch.cuda.synchronize()
        ctx.generation = inst.diff_forward(Time, BoxSize, grid.detach(), out, N, pnu, store_intervals=not recompute)
        ctx.inst = inst
        ctx.recompute = recompute
        ctx.mass_device = masses.device
        ctx.hist_shape = tuple(history.shape)
        ctx.save_for_backward(grid)
        return out, pnu

    @staticmethod
    def backward(ctx, gout, gpnu):
        (grid,) = ctx.saved_tensors
        if gout is None:
            gout = torch.zeros_like(grid)
        if gpnu is None:
            gpnu = torch.zeros(ctx.hist_shape[0], dtype=torch.float64, device=grid.device)
        gout = gout.contiguous()
        gpnu = gpnu.contiguous().to(torch.float64)
        gin = torch.empty_like(grid)
        Dbar = torch.empty(ctx.hist_shape, dtype=torch.float64, device=grid.device)
        torch.cuda.synchronize()
        mbar = ctx.inst.diff_backward(gout, grid.detach(), gpnu, gin, Dbar, recompute=ctx.recompute,
                                      generation=ctx.generation)
        return (gin, Dbar, torch.as_tensor(mbar, dtype=torch.float64, device=ctx.mass_device), None, None, None,
                None, None)


class NeutrinoStep:
    def __init__(self, instance, scalefact, Time, BoxSize, recompute=False):
        self.inst = instance
        self.scalefact = np.ascontiguousarray(scalefact, dtype=np.float64)
        self.Time = Time
        self.BoxSize = BoxSize
        self.recompute = recompute

    def __call__(self, grid, history, masses):
        return _Fn.apply(grid, history, masses, self.inst, self.scalefact, self.Time, self.BoxSize, self.recompute)
