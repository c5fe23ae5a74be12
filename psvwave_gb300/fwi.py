"""Full-waveform inversion drivers over the GPU gradient.

The reference's typical workflow (docs-source/source/typical-workflow.rst:
19-75; Notebook 2, cells 15-17) wraps an fdModel in a small class whose
`misfit(m)` and `grad(m)` share one gradient computation per model vector
(cached on the last vector, compared with numpy.allclose), optionally
smooths the gradient with a Gaussian filter per parameter, and hands both
to scipy.optimize.minimize with method "L-BFGS-B". `FWI` is that class,
`lbfgs` that call; the gradient runs on the GPU:

* mode "reference": the reference's gradient, run_model (all shots
  forward with snapshots, misfit, adjoint sources, kernel reset, all shots
  adjoint, velocity mapping; src/fdModel.cpp:1291-1308) and
  get_gradient_vector (block sums over the free region,
  src/fdModel.cpp:1358-1515);
* mode "exact": the exact discrete adjoint (fdModel.exact_gradient, with
  checkpoints every `checkpoint_every` steps), summed over the same blocks.
"""
import numpy as np


def gradient_vector(model, g_vp, g_vs, g_rho):
    """Fields [nx][nz] of d(misfit)/d(vp, vs, rho) as a gradient in the
    model-vector basis: sums over npx x npz blocks of the free region,
    block (bx, bz) at index bx + bz * nx_free_parameters / npx, vector
    [vp | vs | rho] (the layout of get_gradient_vector,
    src/fdModel.cpp:1358-1515)."""
    npx, npz = model.npx, model.npz
    bx, bz = model.nx_free_parameters // npx, model.nz_free_parameters // npz
    x0 = model.np_boundary + model.nx_inner_boundary
    z0 = model.np_boundary + model.nz_inner_boundary
    parts = []
    for g in (g_vp, g_vs, g_rho):
        sub = np.asarray(g, dtype=np.float64)[x0:x0 + bx * npx, z0:z0 + bz * npz]
        blocks = sub.reshape(bx, npx, bz, npz).sum(axis=(1, 3))  # [bx][bz]
        parts.append(blocks.T.reshape(-1))                         # bx fastest
    return np.concatenate(parts)


def _smooth(g, model, sigma):
    from scipy.ndimage import gaussian_filter

    shape = (model.nz_free_parameters // model.npz, model.nx_free_parameters // model.npx)
    return np.hstack([gaussian_filter(part.reshape(shape), sigma=sigma).reshape(-1)
                      for part in np.split(g, 3)])


class FWI:
    """Misfit and gradient of an fdModel as functions of its model vector,
    computed together once per vector (the reference workflow's `_fwi`).
    `evaluations` counts gradient computations; `history` holds
    (misfit, max |gradient|) per computation and `iterates` the misfit at
    each accepted L-BFGS-B iterate."""

    def __init__(self, model, smoothing=None, mode="reference", checkpoint_every=100):
        if mode not in ("reference", "exact"):
            raise ValueError("mode must be 'reference' or 'exact'")
        self.model = model
        self.smoothing = smoothing
        self.mode = mode
        self.checkpoint_every = checkpoint_every
        self.last_model = None
        self._misfit = None
        self.g = None
        self.evaluations = 0
        self.history = []
        self.iterates = []
        self._seen = []  # (vector, misfit) of every computation

    def _compute(self, m):
        model = self.model
        model.set_model_vector(m)
        if self.mode == "reference":
            model.run_model(False, True)
            mis = model.misfit
            g = model.get_gradient_vector()
        else:
            mis, fields = model.exact_gradient(self.checkpoint_every)
            g = gradient_vector(model, *fields)
        if self.smoothing is not None:
            g = _smooth(g, model, self.smoothing)
        self._misfit, self.g = float(mis), g
        self.last_model = np.array(m, dtype=np.float64, copy=True)
        self.evaluations += 1
        self.history.append((self._misfit, float(np.abs(g).max())))
        self._seen.append((self.last_model, self._misfit))

    def misfit_at(self, m):
        """The misfit of an already evaluated vector (None if there is none)."""
        for v, f in reversed(self._seen):
            if np.allclose(m, v):
                return f
        return None

    def _fresh(self, m):
        return self.last_model is not None and np.allclose(m, self.last_model)

    def misfit(self, m):
        if not self._fresh(m):
            self._compute(m)
        return self._misfit

    def grad(self, m):
        if not self._fresh(m):
            self._compute(m)
        return self.g


def lbfgs(model, m0=None, smoothing=None, mode="reference", checkpoint_every=100, maxiter=50,
          gtol=1e-6, maxcor=10, callback=None):
    """L-BFGS-B over the model vector from m0 (default: the model's current
    vector), with the reference notebook's options (gtol 1e-6, maxcor 10).
    Returns (scipy OptimizeResult, FWI); the model is left at the last
    evaluated vector."""
    from scipy.optimize import minimize

    problem = FWI(model, smoothing=smoothing, mode=mode, checkpoint_every=checkpoint_every)
    x0 = model.get_model_vector() if m0 is None else np.asarray(m0, dtype=np.float64)

    def on_iterate(xk):
        problem.iterates.append(problem.misfit_at(xk))
        if callback is not None:
            callback(xk)

    res = minimize(problem.misfit, x0, method="L-BFGS-B", jac=problem.grad, callback=on_iterate,
                   options={"gtol": gtol, "maxiter": maxiter, "maxcor": maxcor})
    return res, problem
