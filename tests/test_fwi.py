"""FWI drivers (psvwave_gb300.fwi) on CPU: the gradient-vector basis of the
exact mode against the oracle's own get_gradient_vector, and the L-BFGS-B
driver's caching on a quadratic stand-in for a model."""
import numpy as np

from psvwave_gb300 import fwi
from tests.conftest import SMALL_INI


def test_gradient_vector_matches_the_model_vector_basis(golden):
    """Block sums of velocity kernels over the free region, in the layout
    of get_gradient_vector (src/fdModel.cpp:1358-1515), at npx = npz = 2."""
    from oracle.portbind import OracleModel

    o = OracleModel(SMALL_INI)
    o.set_parameter_fields(*golden["target"])
    for s in range(o.n_shots):
        o.forward_simulate(s, False)
    o.set_observed_data(*o.get_synthetic_data())
    o.set_parameter_fields(*golden["start"])
    o.run_model(True)
    ref = o.get_gradient_vector()
    got = fwi.gradient_vector(o, *o.get_kernels())
    assert got.shape == ref.shape
    assert np.allclose(got, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())


class _Quadratic:
    """f(m) = 0.5 |m - m*|^2 with the fdModel calls the L-BFGS-B loop makes."""

    def __init__(self, n, seed=0):
        rng = np.random.default_rng(seed)
        self.target = rng.standard_normal(n)
        self.m = np.zeros(n)
        self.runs = 0
        self.misfit = None

    def get_model_vector(self):
        return self.m.copy()

    def set_model_vector(self, m):
        self.m = np.array(m, dtype=np.float64)

    def run_model(self, verbose=False, simulate_adjoint=True):
        self.runs += 1
        self.misfit = 0.5 * float(np.sum((self.m - self.target) ** 2))

    def get_gradient_vector(self):
        return self.m - self.target


def test_lbfgs_driver_converges_and_computes_each_vector_once():
    q = _Quadratic(50)
    res, problem = fwi.lbfgs(q, maxiter=20, gtol=1e-10)
    assert res.fun < 1e-12
    assert np.allclose(res.x, q.target, atol=1e-6)
    # misfit and grad at the same vector share one computation.
    assert problem.evaluations == q.runs == res.nfev
    assert [h[0] for h in problem.history][0] == 0.5 * float(np.sum(q.target ** 2))


class _Blocks(_Quadratic):
    """The quadratic stand-in with the model-vector geometry attributes:
    12 x 8 free cells, one point per block, vector [vp | vs | rho]."""

    nx_free_parameters, nz_free_parameters, npx, npz = 12, 8, 1, 1

    def __init__(self):
        super().__init__(3 * 12 * 8)


def test_gradient_smoothing_follows_the_model_vector_layout():
    """With smoothing, each parameter's block of the gradient is filtered as
    an image of nz_free x nx_free (index bx + bz * nx_free, the reference
    workflow's reshape): a gradient concentrated at one block spreads
    symmetrically in x and z around it, and stays within its parameter."""
    q = _Blocks()
    bx, bz, nxb = 5, 3, 12
    q.target[:] = 0.0
    q.m = np.zeros_like(q.target)
    q.m[96 + bx + bz * nxb] = 1.0  # vs block, one cell
    g = fwi.FWI(q, smoothing=1.0).grad(q.m)
    vp, vs, rho = np.split(g, 3)
    assert not vp.any() and not rho.any()
    img = vs.reshape(8, 12)
    assert np.unravel_index(np.argmax(img), img.shape) == (bz, bx)
    assert np.isclose(img[bz, bx - 1], img[bz, bx + 1])
    assert np.isclose(img[bz - 1, bx], img[bz + 1, bx])
    assert np.isclose(img[bz, bx + 1], img[bz + 1, bx])  # isotropic filter
    assert np.isclose(img.sum(), 1.0)
