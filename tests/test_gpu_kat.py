"""The reference's own known-answer tests run through the GPU path, at the
reference's tolerances (and at the tighter bounds the oracle reaches)."""
import pytest

import kat

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,tight", [
    ("constvel2D", 2e-8), ("timedependentvel2D", 1e-10), ("diffusion2D", 1e-9), ("hyperdiffusion", 1e-9),
])
@pytest.mark.parametrize("stepper", ["RK4", "ETDRK4"])
def test_reference_kat_2d_gpu(gpu, name, tight, stepper):
    err, rtol = getattr(kat, name)(gpu, gpu.GPU(), stepper=stepper)
    assert err <= rtol, f"{name}: {err:.3e} > reference rtol {rtol:.3e}"
    assert err <= tight


@pytest.mark.parametrize("name,tight", [("constvel1D", 1e-9), ("timedependentvel1D", 1e-9), ("diffusion1D", 1e-9)])
@pytest.mark.parametrize("stepper", ["RK4", "ETDRK4"])
def test_reference_kat_1d_gpu(gpu, name, tight, stepper):
    err, rtol = getattr(kat, name)(gpu, gpu.GPU(), stepper=stepper)
    assert err <= rtol, f"{name}: {err:.3e} > reference rtol {rtol:.3e}"
    assert err <= tight


def test_diffusion1D_timevarying_gpu(gpu):
    err, rtol = kat.diffusion1D(gpu, gpu.GPU(), steadyflow=False)
    assert err <= rtol and err <= 1e-9


def test_diffusion2D_timevarying_gpu(gpu):
    err, rtol = kat.diffusion2D(gpu, gpu.GPU(), steadyflow=False)
    assert err <= rtol and err <= 1e-9


@pytest.mark.parametrize("name,tight", [("constvel3D", 2e-8), ("timedependentvel3D", 1e-10)])
def test_reference_kat_3d_gpu(gpu, name, tight):
    err, rtol = getattr(kat, name)(gpu, gpu.GPU(), n=128)  # the reference's 128³
    assert err <= rtol and err <= tight


@pytest.mark.parametrize("steadyflow", [True, False])
def test_reference_kat_diffusion3D_gpu(gpu, steadyflow):
    err, rtol = kat.diffusion3D(gpu, gpu.GPU(), steadyflow=steadyflow)
    assert err <= rtol and err <= 4.1e-4


@pytest.mark.parametrize("stepper,tight", [("RK4", 1e-9), ("ETDRK4", 1e-11)])
def test_reference_kat_diffusion_multilayerqg_gpu(gpu, stepper, tight):
    """test_diffusion_multilayerqg through Problem(MQGprob; ...) (the layers
    are the solves of one batched handle)."""
    err, rtol = kat.diffusion_multilayerqg(gpu, gpu.GPU(), stepper=stepper)
    assert err <= rtol and err <= tight
