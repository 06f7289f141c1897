"""The differentiable lens (configuration 4): forward against the reference's
trace and the plain FP64 tracer, adjoint gradient against central finite
differences (of the lens forward and of the FP64 tracer) and through
torch.autograd."""
import numpy as np
import pytest

from helpers import NS, load_case
from raypier_optics_gb300 import ctracer, lens, tracer
from raypier_optics_gb300 import workloads as W

pytestmark = pytest.mark.gpu

# gradient tolerance: |adjoint - FD| <= GRAD_RTOL |FD| + GRAD_ATOL_REL * max |FD|
GRAD_RTOL = 1e-4
GRAD_ATOL_REL = 1e-7


def rms(xy):
    d = xy - xy.mean(axis=0)
    return float(np.sqrt(np.mean(np.sum(d * d, axis=1))))


def image_from_trace(gens, n_surf):
    """Image-plane points of a trace of config4_spec: the last generation's
    rays end on the image plane."""
    g = gens[n_surf]
    return g["origin"] + g["direction"] * g["length"][:, None], g["parent_idx"]


def test_lens_forward_matches_reference_trace():
    case = load_case("config4_sub64")
    rays, gens = case["rays"], case["gens"]
    C = W.CONFIG4
    L = lens.Lens(W.LENS4_SEMI, W.LENS4_INDEX, rays, max_length=C["max_length"], atol=C["atol"],
                  tolerance=C["tolerance"])
    loss, nv = L.forward(W.config4_params())
    xy, valid = L.image()
    ref, _ = image_from_trace(gens, len(W.LENS4_SEMI))
    assert nv == len(rays) == len(ref) and valid.all()
    np.testing.assert_allclose(xy, ref[:, :2], rtol=1e-9, atol=1e-12)
    assert loss == pytest.approx(rms(ref[:, :2]), rel=1e-9)
    L.close()


def test_lens_forward_equals_the_fp64_tracer():
    n = 4096
    L = lens.config4_lens(n_rays=n)
    p = W.config4_params()
    loss, nv = L.forward(p)
    xy, valid = L.image()
    rays, wl = W.config4_rays(ctracer.ray_dtype, n)
    rc = ctracer.RayCollection.from_array(rays)
    rc.wavelengths = wl
    traced, _ = tracer.trace_rays(rc, W.build_scene(W.config4_spec(p), NS), recursion_limit=10,
                                  max_length=W.CONFIG4["max_length"], flags=tracer.RP_TRACE_PLAIN_FP64)
    gens = [t.copy_as_array() for t in traced]
    img, parent = image_from_trace(gens, len(W.LENS4_SEMI))
    assert valid.all() and len(img) == n
    np.testing.assert_array_equal(xy, img[:, :2])
    assert loss == rms(img[:, :2]) or loss == pytest.approx(rms(img[:, :2]), rel=1e-13)
    L.close()


@pytest.fixture(scope="module")
def full_lens():
    L = lens.config4_lens()
    yield L
    L.close()


def test_adjoint_matches_central_differences(full_lens):
    p = W.config4_params()
    loss, nv = full_lens.forward(p)
    assert nv == W.CONFIG4["n_rays"] and 0.0 < loss < 1.0
    g = full_lens.backward()
    fd = lens.central_differences(full_lens, p, rel_step=W.CONFIG4["fd_step"])
    fd = np.array([fd[j] for j in range(len(p))])
    err = np.abs(g - fd)
    bound = GRAD_RTOL * np.abs(fd) + GRAD_ATOL_REL * np.max(np.abs(fd))
    print("loss", loss, "max rel err", float(np.max(err / np.maximum(np.abs(fd), 1e-300))))
    assert np.all(err <= bound), list(zip(np.flatnonzero(err > bound), g[err > bound], fd[err > bound]))


def test_adjoint_matches_differences_of_the_fp64_tracer():
    """Central differences of the loss computed from the general FP64 tracer
    (rp_trace_rays on the lens as an ordinary scene) against the adjoint."""
    n = 2048
    L = lens.config4_lens(n_rays=n)
    p = W.config4_params()
    L.forward(p)
    g = L.backward()
    rays, wl = W.config4_rays(ctracer.ray_dtype, n)

    def loss_tracer(params):
        rc = ctracer.RayCollection.from_array(rays)
        rc.wavelengths = wl
        traced, _ = tracer.trace_rays(rc, W.build_scene(W.config4_spec(params), NS), recursion_limit=10,
                                      max_length=W.CONFIG4["max_length"], flags=tracer.RP_TRACE_PLAIN_FP64)
        img, _ = image_from_trace([t.copy_as_array() for t in traced], len(W.LENS4_SEMI))
        return rms(img[:, :2])

    for j in (0, 5, 9, 17, 26, 33, 39):  # curvatures, conics, A4, A6, thicknesses
        h = W.CONFIG4["fd_step"] * abs(p[j])
        pp, pm = p.copy(), p.copy()
        pp[j] += h
        pm[j] -= h
        fd = (loss_tracer(pp) - loss_tracer(pm)) / (pp[j] - pm[j])
        assert abs(g[j] - fd) <= 1e-4 * abs(fd) + 1e-9, (j, g[j], fd)
    L.close()


def test_torch_autograd_function(full_lens):
    torch = pytest.importorskip("torch")
    p = W.config4_params()
    t = torch.tensor(p, dtype=torch.float64, requires_grad=True)
    loss = lens.spot_rms(full_lens, t)
    loss.backward()
    value = loss.detach().item()
    assert value == pytest.approx(full_lens.forward(p)[0], rel=0, abs=0)
    np.testing.assert_array_equal(t.grad.numpy(), full_lens.backward())
    # one descent step lowers the loss
    with torch.no_grad():
        step = t - 1e-3 * value * t.grad / torch.linalg.norm(t.grad) * torch.abs(t)
    assert lens.spot_rms(full_lens, step).item() < value
