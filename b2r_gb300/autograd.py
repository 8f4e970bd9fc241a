"""torch.autograd face of the elastic-wave adjoint (checking aid).

``EqwpMisfit.apply(lam, mu, rho, problem)`` returns the receiver misfit
J = 1/2 |d_syn - d_obs|^2 of the staggered elastic-wave model as a 0-d
tensor; its backward returns dJ/dlambda, dJ/dmu, dJ/drho from the library's
hand-written discrete adjoint (b2r_eqwp_misfit_gradient).  lam, mu, rho are
env-shaped (z, y, x) CPU tensors of the interior cells; the fixed shell takes
the edge values.  Used by the tests to compare with central finite
differences; the computation itself runs entirely in libb2r.
"""
import numpy as np
import torch

from . import MODEL_EQWP_STAG, MODEL_HEAT, Domain


def _padded(a, H):
    return np.pad(np.asarray(a, np.float64), H, mode="edge")


class EqwpMisfit(torch.autograd.Function):
    @staticmethod
    def forward(ctx, lam, mu, rho, problem):
        P = problem
        env = P["env"]
        with Domain(MODEL_EQWP_STAG, env, D=2, R=1, dt=P["dt"], h=P["h"], src=P["src"]) as d:
            H = d.halo - 2          # the domain array's shell is D = 2 deep
            shell = 2
            mats = [lam.detach().cpu().numpy(), mu.detach().cpu().numpy(),
                    1.0 / rho.detach().cpu().numpy()]
            for name, m in zip(("lambda", "mu", "buoy"), mats):
                d.upload(np.ascontiguousarray(_padded(m, shell), np.float32), field=name)
            zero = np.zeros(d.domain_shape, np.float32)
            for k in range(9):
                d.upload(zero, field=k)
            d.set_source(P["amps"])
            J, g, _ = d.eqwp_misfit_gradient(P["nsteps"], P["rec"], P["d_obs"],
                                             P.get("ckpt_every", 50))
            del H
        ctx.save_for_backward(*[torch.from_numpy(x) for x in g])
        return torch.tensor(J, dtype=torch.float64)

    @staticmethod
    def backward(ctx, gJ):
        gl, gm, gr = ctx.saved_tensors
        return gJ * gl, gJ * gm, gJ * gr, None


class HeatMisfit(torch.autograd.Function):
    """``HeatMisfit.apply(kappa, problem)``: receiver misfit of the
    conductivity-scaled heat scheme (b2r_heat_record) as a 0-d tensor, with
    dJ/dkappa from the library's discrete adjoint (b2r_heat_misfit_gradient).
    kappa: env-shaped (z, y, x) CPU tensor of the interior cells; problem:
    dict with env, D, coef (alpha_dt, dx, dy, dz), u0 (domain array with its
    D-deep shell), nsteps, rec, d_obs and optionally ckpt_every."""

    @staticmethod
    def forward(ctx, kappa, problem):
        P = problem
        a, dx, dy, dz = P["coef"]
        with Domain(MODEL_HEAT, P["env"], D=P["D"], R=1, alpha_dt=a, dx=dx, dy=dy, dz=dz) as d:
            d.upload(np.ascontiguousarray(_padded(kappa.detach().cpu().numpy(), P["D"]), np.float32),
                     field="kappa")
            d.upload(np.ascontiguousarray(P["u0"], np.float32))
            J, g, _ = d.heat_misfit_gradient(P["nsteps"], P["rec"], P["d_obs"], P.get("ckpt_every", 50))
        ctx.save_for_backward(torch.from_numpy(g))
        return torch.tensor(J, dtype=torch.float64)

    @staticmethod
    def backward(ctx, gJ):
        (g,) = ctx.saved_tensors
        return gJ * g, None
