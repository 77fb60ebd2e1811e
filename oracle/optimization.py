"""numpy restatement of the reference's optimiser updates.

TEST INFRASTRUCTURE ONLY: imported by ``tests/`` to check the device
optimiser steps (``qg_adam_step``, ``qg_gd_step``, ``qg_plateau_step``).
The ``qradient_gb300`` product never imports this module.

Each class follows ``qradient/optimization.py`` line by line, with the same
numpy expressions in the same order, so its results are bit-identical to the
reference's; the tests pin that against golden trajectories the reference's
own classes produced (``tests/golden/make_golden.py --optimizer``).
"""
import numpy as np


class Adam:
    """optimization.py:151-167."""

    def __init__(self, parameters, step_size=0.001, beta1=0.9, beta2=0.999, eps=10.0 ** -8):
        self.parameters = np.array(parameters, dtype=np.float64)
        self.step_size, self.beta1, self.beta2, self.eps = step_size, beta1, beta2, eps
        self.m = np.zeros(self.parameters.shape)
        self.v = np.zeros(self.parameters.shape)
        self.iter = 0

    def step(self, gradient, *args):
        self.iter += 1  # :162
        self.m = self.beta1 * self.m + (1 - self.beta1) * gradient  # :163
        self.v = self.beta2 * self.v + (1 - self.beta2) * gradient ** 2  # :164
        m_hat = self.m / (1 - self.beta1 ** self.iter)  # :165
        v_hat = self.v / (1 - self.beta2 ** self.iter)  # :166
        self.parameters -= self.step_size * m_hat / (np.sqrt(v_hat) + self.eps)  # :167


class GradientDescent:
    """optimization.py:169-175."""

    def __init__(self, parameters, step_size=0.001, decay_function=None):
        self.parameters = np.array(parameters, dtype=np.float64)
        self.step_size = step_size
        self.decay_function = decay_function or (lambda s, i: s)
        self.iter = 0

    def step(self, gradient, *args):
        self.iter += 1
        self.parameters -= self.decay_function(self.step_size, self.iter) * gradient  # :175


class RateDecayOnPlateau:
    """optimization.py:177-194."""

    def __init__(self, parameters, step_size=0.001, plateau_length=10, decay_rate=0.5):
        self.parameters = np.array(parameters, dtype=np.float64)
        self.step_size = step_size
        self.plateau_length = plateau_length
        self.decay_rate = decay_rate
        self.plateau_counter = 0
        self.cost = 10.0 ** 10
        self.iter = 0

    def step(self, gradient, new_cost):
        self.iter += 1
        if new_cost > self.cost:  # :186-190
            self.plateau_counter += 1
            if self.plateau_counter >= self.plateau_length:
                self.step_size *= self.decay_rate
                self.plateau_counter = 0
        else:  # :191-193
            self.cost = new_cost
            self.plateau_counter = 0
        self.parameters -= self.step_size * gradient  # :194
