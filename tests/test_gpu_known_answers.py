"""A known answer of the reference's own tests on the device: the analytic
Gaussian of tests/test_vertical_diffusion.F90 (a Gaussian of amplitude 5 and
width 5 m in a 100 m column of 100 layers, constant diffusivity 0.1 m2/s,
200 steps of 5 s) through the FP64 column solve and both float solves of the
mixed form (float storage, FP64 storage with float increments).

Tolerances: against the analytic solution 1.5e-3 of the amplitude (the
oracle's own discretisation error is 7e-4); against the oracle 1e-12 for the
FP64 form, 1e-5 (FP64 storage) and 5e-5 (float storage) for the float
solves; column totals conserved to 1e-13 (FP64), 1e-6 and 1e-4."""

import numpy as np
import pytest

from tests.test_oracle_vertical_diffusion import GAUSS, gaussian_column

pytestmark = pytest.mark.gpu

TOL = {"fp64": (1e-12, 1e-13), "float64_storage": (1e-5, 1e-6), "float32": (5e-5, 1e-4)}


def _device(form):
    def run(make_diffusion, Th, hn, nuh, var, cnpar, dt, nstep):
        import torch

        from getm_gb300 import operators
        from getm_gb300.core import Array, CENTERS, INTERFACES, make_grids

        Td = make_grids(Th)
        Td.hn.all_values.copy_(torch.from_numpy(hn))
        solve = torch.float64 if form == "fp64" else torch.float32
        store = torch.float32 if form == "float32" else torch.float64
        vd = operators.VerticalDiffusion(Td, cnpar)
        nuh_d = Array(Td, torch.from_numpy(nuh).to(device=Td.device, dtype=solve), z=INTERFACES)
        v = Array(Td, torch.from_numpy(var).to(device=Td.device, dtype=store), z=CENTERS)
        for _ in range(nstep):
            vd(nuh_d, dt, v)
        torch.cuda.synchronize()
        return v.all_values.double().cpu().numpy()

    return run


@pytest.mark.parametrize("form", ["fp64", "float64_storage", "float32"])
@pytest.mark.parametrize("cnpar", [0.5, 1.0])
def test_gaussian_against_the_analytic_solution(form, cnpar):
    from oracle import oracle as O

    _, var_o, _, _, _ = gaussian_column(O.VerticalDiffusion, cnpar)
    wet, var, ana, total0, total = gaussian_column(None, cnpar, to_device=_device(form), from_device=lambda x: x)
    cmax = GAUSS["cmax"]
    e_ana = np.abs(var[:, wet] - ana[:, None]).max() / cmax
    e_oracle = np.abs(var[:, wet] - var_o[:, wet]).max() / cmax
    e_total = np.abs(total - total0).max() / total0.max()
    print(f"gaussian {form} cnpar={cnpar}: analytic {e_ana:.2e} oracle {e_oracle:.2e} total {e_total:.2e}")
    assert e_ana < 1.5e-3
    assert e_oracle < TOL[form][0]
    assert e_total < TOL[form][1]
