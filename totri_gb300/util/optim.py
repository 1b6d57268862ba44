"""Learning-rate schedules and the optimiser wrapper of the fitting loops.

Behaviour the fitting loops rely on (the reference's totri/util/optim.py:14-95
offers the same schedules under the names kept below as constructors):

* A schedule maps the iteration count i = 0, 1, 2, ... to a learning rate:
  - constant: the same value for every i;
  - linear: ``start`` at i = 0 moving evenly to ``end`` at i = n - 1, and held
    at the nearer end outside that range;
  - geometric approach: a value that moves the fraction (1 - gamma) of its
    remaining distance towards ``target`` each time it is queried, whatever i.
* ``TotriOptimizer`` runs Adam or SGD over one parameter group. It draws a
  rate when it is given parameters (at construction and on every
  ``set_params``) and a new one after each ``step``. A warm-up of w draws
  follows each ``set_params``: its k-th draw (k = 0 .. w-1) is the schedule's
  rate scaled by ((k + 1) / (w + 1))^2.
"""
import torch


class Schedule:
    """A learning-rate schedule (see the module docstring); call it with the
    iteration count."""

    def __init__(self, kind, **params):
        if kind not in ("constant", "linear", "approach"):
            raise ValueError("unknown schedule kind %r" % (kind,))
        self.kind = kind
        self.params = params

    def __call__(self, iteration):
        p = self.params
        if self.kind == "constant":
            return p["value"]
        if self.kind == "linear":
            t = iteration / (p["n"] - 1)
            t = 0.0 if t < 0.0 else (1.0 if t > 1.0 else t)
            return p["start"] + t * (p["end"] - p["start"])
        p["value"] = p["target"] + p["gamma"] * (p["value"] - p["target"])
        return p["value"]


# The reference's schedule names, as constructors of the same schedules.
Interpolator = Schedule


def ConstantInterpolator(constant):  # noqa: N802
    return Schedule("constant", value=constant)


def LinearInterpolator(value_0, value_n, n):  # noqa: N802
    return Schedule("linear", start=value_0, end=value_n, n=n)


def MultiplicativeInterpolator(value, target, gamma=0.99):  # noqa: N802
    return Schedule("approach", value=value, target=target, gamma=gamma)


class TotriOptimizer:
    """Adam or SGD whose learning rate follows a schedule (a number means a
    constant rate), with a quadratic warm-up after each parameter reset."""

    _OPTIMISERS = {"Adam": torch.optim.Adam, "SGD": torch.optim.SGD}

    def __init__(self, params, lr_interpolator, warmup=0, optimizer="Adam"):
        if optimizer not in self._OPTIMISERS:
            raise ValueError("Unsupported Optimizer %s" % optimizer)
        self._make = self._OPTIMISERS[optimizer]
        self.schedule = (lr_interpolator if callable(lr_interpolator)
                         else ConstantInterpolator(lr_interpolator))
        self.iteration = 0
        self.lr = None
        self.set_params(params, warmup)

    def _draw(self):
        rate = self.schedule(self.iteration)
        self.iteration += 1
        if self._warm_left > 0:
            done = self._warmup - self._warm_left
            rate *= ((done + 1) / (self._warmup + 1)) ** 2
            self._warm_left -= 1
        self.lr = rate
        return rate

    def set_params(self, params, warmup=0):
        """Starts a new optimiser over `params` (fresh moments) and a new warm-up."""
        self._warmup = self._warm_left = warmup
        self.optim = self._make(params, self._draw())

    def zero_grad(self):
        self.optim.zero_grad()

    def step(self):
        self.optim.step()
        rate = self._draw()
        for group in self.optim.param_groups:
            group["lr"] = rate
