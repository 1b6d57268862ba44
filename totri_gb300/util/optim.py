"""Learning-rate schedules and the Adam/SGD wrapper the fitting loops use
(reference totri/util/optim.py:14-95).

An interpolator maps the iteration to a learning rate: constant, linear from
value_0 to value_n over n iterations, or multiplicative (each call moves the
value a fraction 1 - gamma towards the target, ignoring the iteration).
``TotriOptimizer`` takes the first rate at construction and a new one after
every step; during a warm-up of w steps the rate is scaled by
((k + 1) / (w + 1))^2 at the k-th rate drawn.
"""
import torch


class Interpolator:
    pass


class ConstantInterpolator(Interpolator):
    def __init__(self, constant):
        self.constant = constant

    def __call__(self, _):
        return self.constant


class LinearInterpolator(Interpolator):
    def __init__(self, value_0, value_n, n):
        self.value_0, self.value_n, self.n = value_0, value_n, n

    def __call__(self, i):
        w = max(min(i / (self.n - 1), 1), 0)
        return (1 - w) * self.value_0 + w * self.value_n


class MultiplicativeInterpolator(Interpolator):
    def __init__(self, value, target, gamma=0.99):
        self.value, self.target, self.gamma = value, target, gamma

    def __call__(self, _):
        self.value = self.gamma * self.value + (1 - self.gamma) * self.target
        return self.value


class TotriOptimizer:
    def __init__(self, params, lr_interpolator, warmup=0, optimizer="Adam"):
        if optimizer not in ("Adam", "SGD"):
            raise ValueError("Unsupported Optimizer %s" % optimizer)
        self.iteration = 0
        self.optim_type = optimizer
        self.lr = None
        if not isinstance(lr_interpolator, Interpolator):
            lr_interpolator = ConstantInterpolator(lr_interpolator)
        self.lr_interpolator = lr_interpolator
        self.set_params(params, warmup)

    def set_params(self, params, warmup=0):
        self.set_warmup(warmup)
        lr = self.get_next_lr()
        cls = torch.optim.Adam if self.optim_type == "Adam" else torch.optim.SGD
        self.optim = cls(params, lr)

    def set_warmup(self, warmup):
        self.warmup_iter = 0
        self.warmup_total = warmup

    def zero_grad(self):
        self.optim.zero_grad()

    def get_next_lr(self):
        self.lr = self.lr_interpolator(self.iteration)
        if self.warmup_total > 0 and self.warmup_iter < self.warmup_total:
            self.lr *= ((self.warmup_iter + 1) / (self.warmup_total + 1)) ** 2
            self.warmup_iter += 1
        self.iteration += 1
        return self.lr

    def step(self):
        self.optim.step()
        lr = self.get_next_lr()
        for group in self.optim.param_groups:
            group["lr"] = lr
