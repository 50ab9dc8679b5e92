"""Failure paths of the entry points: every bad request comes back as a
status (FameError on the Python side) with the plan still usable; nothing
faults or waits on the GPU."""
import ctypes as C

import numpy as np
import pytest
import torch

import fame
from fame import _lib as L

pytestmark = pytest.mark.gpu


@pytest.fixture
def plan():
    p = fame.woodpile_plan(6, [fame.fcc_point("X"), fame.fcc_point("L")])
    yield p
    p.close()


def test_gradient_needs_field_plan(cuda, fame_lib, plan):
    ev = torch.zeros((1, 4 * plan.Nq), dtype=torch.complex128, device="cuda")
    with pytest.raises(fame.FameError) as e:
        plan.eig_gradient(ev, [1.0])
    assert e.value.code == L.FAME_ERR_UNSUPPORTED
    with pytest.raises(fame.FameError) as e:
        plan.set_fields(np.ones(plan.Nq), np.zeros(plan.Nq))
    assert e.value.code == L.FAME_ERR_BAD_ARG


def test_field_plan_rejects_non_definite_medium(cuda, fame_lib):
    n = 4
    th = np.stack([fame.bloch_angles(fame.fcc_point("X"))])
    eps = np.full(n ** 3, 2.0)
    gam = np.full(n ** 3, 2.0)  # eps - gamma^2 < 0
    with pytest.raises(fame.FameError) as e:
        fame.Plan.from_fields(n, th, eps, gam)
    assert e.value.code == L.FAME_ERR_BAD_ARG


def test_restore_and_solver_arguments(cuda, fame_lib, plan):
    lib = fame.load()
    ev = torch.zeros((1, 4 * plan.Nq), dtype=torch.complex128, device="cuda")
    with pytest.raises(fame.FameError) as e:
        plan.restore(ev, [1.0], inst=[5])  # instance out of range
    assert e.value.code == L.FAME_ERR_BAD_ARG
    assert lib.fame_autotune(plan.raw, 7, 2, None, None, None) == L.FAME_ERR_BAD_ARG
    assert lib.fame_set_tune(plan.raw, L.FAME_C64, 2, 0, 100) == L.FAME_ERR_BAD_ARG
    ew = np.zeros(1)
    assert lib.fame_jdsira(plan.raw, L.FAME_C64, 0, 0, 0.0, 0.0, 1e-8, 20, 4, 1e-2, 100,
                           ew.ctypes.data_as(C.POINTER(C.c_double)), None, None, None) == L.FAME_ERR_BAD_ARG
    assert lib.fame_lanczos(plan.raw, L.FAME_C64, 0, 10, 1e-10, 100, 5, None, 1e-12,
                            ew.ctypes.data_as(C.POINTER(C.c_double)), None, None, None) == L.FAME_ERR_BAD_ARG
    # the plan still works after every refusal
    x = torch.randn(2, 4 * plan.Nq, dtype=torch.complex128, device="cuda")
    y = plan.apply_B(x)
    assert torch.isfinite(y).all()


def test_unsupported_grid_size(cuda, fame_lib):
    with pytest.raises(fame.FameError) as e:
        fame.woodpile_plan(7, [fame.fcc_point("X")])
    assert e.value.code == L.FAME_ERR_UNSUPPORTED
