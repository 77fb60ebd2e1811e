"""Training loops with the parameter update on the GPU (qradient/optimization.py).

``McCleanOpt`` (:41-97) and ``QaoaOpt`` (:99-142) drive ``grad_run`` and an
optimiser (``Adam`` :151-167, ``GradientDescent`` :169-175,
``RateDecayOnPlateau`` :177-194) picked from the same dict
(``{'name': 'Adam', 'step_size': ...}``, :23-39).  Here a step is one
adjoint-gradient launch sequence followed by one update kernel on the same
stream: the gradient, the cost, the moments, the parameters and both
histories stay in device memory, and no value returns to the host unless
the caller reads one.  Every update is bit-identical to the reference's for
the same gradient (explicitly rounded double operations in numpy's order).

Differences from the reference, all in where data lives:

* ``param_history`` / ``cost_history`` read as numpy arrays (a device-to-host
  copy per read); ``param_history_tensor`` / ``cost_history_tensor`` are the
  device tensors themselves.
* ``optimizer.parameters`` is a float64 device tensor, and ``McCleanOpt``
  points ``circuit.angles`` at it, as the reference points ``circuit.angles``
  at the optimiser's array (:91).
* ``RateDecayOnPlateau`` keeps its best cost, plateau counter and step size
  on the device; reading ``step_size`` copies it back.
* Shot-based gradients (``shot_num > 0``) are not on the GPU path and raise
  ``NotImplementedError``.
"""
import torch

from . import _lib, _native

_NAMES = ("Adam", "GradientDescent", "RateDecayOnPlateau")


def _check_optimizer(optimizer):
    name = optimizer.get("name") if isinstance(optimizer, dict) else None
    if name not in _NAMES:
        raise ValueError("No optimizer {} known.".format(optimizer))


def _device_copy(x, device):
    t = torch.as_tensor(x, dtype=torch.float64)
    return t.to(device).clone().contiguous()


def _device_view(x, device, numel):
    """x as a contiguous float64 device tensor, without a copy when it is one."""
    t = torch.as_tensor(x, dtype=torch.float64)
    if t.numel() != numel:
        raise ValueError("expected %d values, got %d" % (numel, t.numel()))
    return t.reshape(-1).to(device, non_blocking=True).contiguous()


def _stream(t):
    return _native.stream_handle(t.device)


# ---------------------------------------------------------------- update rules
class GradientDescentOptimizer:
    """optimization.py:145-149: parameters, step size, iteration count."""

    def init(self, parameters, hyper_parameters, device=None):
        device = _native.require_cuda(device if device is not None else getattr(parameters, "device", None))
        self.parameters = _device_copy(parameters, device)
        self.step_size = hyper_parameters.get("step_size", 0.001)
        self.iter = 0

    @property
    def device(self):
        return self.parameters.device

    def _grad(self, gradient):
        return _device_view(gradient, self.device, self.parameters.numel())


class Adam(GradientDescentOptimizer):
    """optimization.py:151-167; m and v live on the device."""

    def __init__(self, parameters, hyper_parameters, device=None):
        GradientDescentOptimizer.init(self, parameters, hyper_parameters, device)
        self.beta1 = hyper_parameters.get("beta1", 0.9)
        self.beta2 = hyper_parameters.get("beta2", 0.999)
        self.eps = hyper_parameters.get("eps", 10.0 ** -8)
        self.m = torch.zeros_like(self.parameters)
        self.v = torch.zeros_like(self.parameters)

    @property
    def m_hat(self):
        return self.m / (1 - self.beta1 ** self.iter) if self.iter else torch.zeros_like(self.m)

    @property
    def v_hat(self):
        return self.v / (1 - self.beta2 ** self.iter) if self.iter else torch.zeros_like(self.v)

    def step(self, gradient, *args, history_row=None):
        g = self._grad(gradient)
        self.iter += 1
        _lib.check(_lib.load().qg_adam_step(
            _native.ptr(self.parameters), _native.ptr(g), _native.ptr(self.m), _native.ptr(self.v),
            self.parameters.numel(), self.iter, float(self.step_size), float(self.beta1), float(self.beta2),
            float(self.eps), _native.ptr(history_row), _stream(self.parameters)))


class GradientDescent(GradientDescentOptimizer):
    """optimization.py:169-175; the decay function runs on the host."""

    def __init__(self, parameters, hyper_parameters, device=None):
        GradientDescentOptimizer.init(self, parameters, hyper_parameters, device)
        self.decay_function = hyper_parameters.get("decay_function", lambda step_size, iter: step_size)

    def step(self, gradient, *args, history_row=None):
        g = self._grad(gradient)
        self.iter += 1
        lr = float(self.decay_function(self.step_size, self.iter))
        _lib.check(_lib.load().qg_gd_step(_native.ptr(self.parameters), _native.ptr(g), self.parameters.numel(),
                                          lr, _native.ptr(history_row), _stream(self.parameters)))


class RateDecayOnPlateau(GradientDescentOptimizer):
    """optimization.py:177-194 with {best cost, plateau counter, step size}
    in a device array, so the cost the gradient pass wrote is compared on the
    device."""

    def __init__(self, parameters, hyper_parameters, device=None):
        GradientDescentOptimizer.init(self, parameters, hyper_parameters, device)
        self.plateau_length = int(hyper_parameters.get("plateau_length", 10))
        self.decay_rate = hyper_parameters.get("decay_rate", 0.5)
        self._state = torch.tensor([10.0 ** 10, 0.0, float(self._ini_step)], dtype=torch.float64,
                                   device=self.parameters.device)

    @property
    def step_size(self):
        state = getattr(self, "_state", None)
        return self._ini_step if state is None else float(state[2].item())

    @step_size.setter
    def step_size(self, value):
        state = getattr(self, "_state", None)
        if state is None:
            self._ini_step = value
        else:
            state[2] = float(value)

    @property
    def plateau_counter(self):
        return int(self._state[1].item())

    @property
    def cost(self):
        return float(self._state[0].item())

    def step(self, gradient, new_cost, history_row=None):
        g = self._grad(gradient)
        c = _device_view(new_cost, self.device, 1)
        self.iter += 1
        _lib.check(_lib.load().qg_plateau_step(
            _native.ptr(self.parameters), _native.ptr(g), self.parameters.numel(), _native.ptr(c),
            _native.ptr(self._state), self.plateau_length, float(self.decay_rate), _native.ptr(history_row),
            _stream(self.parameters)))


_CLASSES = {"Adam": Adam, "GradientDescent": GradientDescent, "RateDecayOnPlateau": RateDecayOnPlateau}


# ---------------------------------------------------------------- training loops
class ParametrizedCircuitOptimizer:
    """optimization.py:3-39."""

    def init(self, circuit, max_iter):
        self.circuit = circuit
        self.max_iter = int(max_iter)
        self.iter = 0

    def step(self):
        pass

    def reset(self):
        pass

    def pick(self, optimizer, ini_parameters):
        _check_optimizer(optimizer)
        self.optimizer = _CLASSES[optimizer["name"]](ini_parameters, optimizer)

    def __str__(self):
        return self.optimizer_info.__str__()

    @property
    def param_history(self):
        return self.param_history_tensor.cpu().numpy()

    @property
    def cost_history(self):
        return self.cost_history_tensor.cpu().numpy()

    def _check_shots(self, shot_num):
        if shot_num != 0:
            raise NotImplementedError("shot-based gradients (sample_grad*) are not part of the GB300 path; "
                                      "use shot_num=0 for the exact adjoint gradient")

    def _advance(self, grad_fn):
        """One step with the reference's bookkeeping (optimization.py:70-91):
        past the history's end the cost write (iter == max_iter) or the
        parameter-history write (iter + 1 == max_iter) raises IndexError at
        the point where the reference's numpy assignment does."""
        if self.iter >= self.max_iter:
            print("Maximum amount of iterations reached: {}.".format(self.max_iter))
        if self.iter >= self.max_iter:
            grad_fn(None)
            raise IndexError("index {} is out of bounds for axis 0 with size {}".format(self.iter, self.max_iter))
        e = self.cost_history_tensor[self.iter:self.iter + 1]
        g = grad_fn(e)
        last = self.iter + 1 >= self.max_iter
        self.optimizer.step(g, e, history_row=None if last else self.param_history_tensor[self.iter + 1])
        self.iter += 1
        if last:
            raise IndexError("index {} is out of bounds for axis 0 with size {}".format(self.iter, self.max_iter))


class McCleanOpt(ParametrizedCircuitOptimizer):
    """optimization.py:41-97."""

    def __init__(self, circuit, optimizer, max_iter=1000, **kwargs):
        _check_optimizer(optimizer)
        ParametrizedCircuitOptimizer.init(self, circuit, max_iter)
        dev = circuit._device()
        shape = (circuit.lnum, circuit.qnum)
        self.param_history_tensor = torch.zeros((self.max_iter,) + shape, dtype=torch.float64, device=dev)
        self.cost_history_tensor = torch.zeros(self.max_iter, dtype=torch.float64, device=dev)
        ini = kwargs.get("ini_parameters", circuit.angles)
        ini = torch.as_tensor(ini, dtype=torch.float64).to(dev).reshape(shape)
        if self.max_iter > 0:
            self.param_history_tensor[0] = ini
        self.optimizer_info = optimizer
        self.pick(optimizer, ini)
        self.optimizer.parameters = self.optimizer.parameters.reshape(shape)
        self.circuit.angles = self.optimizer.parameters
        self._grad = torch.empty(max(circuit.lnum * circuit.qnum, 1), dtype=torch.float64, device=dev)

    def step(self, shot_num=0, dense_mode=True, component_sampling=False):
        self._check_shots(shot_num)

        def grad_fn(e):
            if e is None:
                e = torch.empty(1, dtype=torch.float64, device=self._grad.device)
            if component_sampling:
                _, g = self.circuit.grad_run_with_component_sampling_tensors(angles=self.optimizer.parameters,
                                                                             out=(e, self._grad))
            else:
                _, g = self.circuit.grad_run_tensors(angles=self.optimizer.parameters, out=(e, self._grad))
            return g

        self._advance(grad_fn)
        self.circuit.angles = self.optimizer.parameters

    def reset(self, **kwargs):
        ini_parameters = kwargs.get("ini_parameters", self.param_history_tensor[0].clone())
        optimizer = kwargs.get("optimizer", self.optimizer_info)
        max_iter = kwargs.get("max_iter", self.max_iter)
        self.__init__(self.circuit, optimizer, max_iter, ini_parameters=ini_parameters)


class QaoaOpt(ParametrizedCircuitOptimizer):
    """optimization.py:99-142; parameters are [p, 2] = (beta, gamma) rows."""

    def __init__(self, circuit, optimizer, betas, gammas, max_iter=1000):
        _check_optimizer(optimizer)
        ParametrizedCircuitOptimizer.init(self, circuit, max_iter)
        dev = circuit._device()
        p = circuit.lnum
        self.param_history_tensor = torch.zeros((self.max_iter, p, 2), dtype=torch.float64, device=dev)
        self.cost_history_tensor = torch.zeros(self.max_iter, dtype=torch.float64, device=dev)
        b = torch.as_tensor(betas, dtype=torch.float64).reshape(-1).to(dev)
        c = torch.as_tensor(gammas, dtype=torch.float64).reshape(-1).to(dev)
        if b.numel() != p or c.numel() != p:
            raise ValueError("Wrong amount of parameters. Expected {} and {}, found {} and {}.".format(
                p, p, b.numel(), c.numel()))
        ini = torch.stack([b, c], dim=1)
        if self.max_iter > 0:
            self.param_history_tensor[0] = ini
        self.optimizer_info = optimizer
        self.pick(optimizer, ini)
        self._grad = torch.empty(max(2 * p, 1), dtype=torch.float64, device=dev)

    def step(self, shot_num=0, dense_mode=True):
        self._check_shots(shot_num)

        def grad_fn(e):
            if e is None:
                e = torch.empty(1, dtype=torch.float64, device=self._grad.device)
            _, g = self.circuit.grad_run_tensors(self.optimizer.parameters, out=(e, self._grad))
            return g

        self._advance(grad_fn)

    def reset(self, **kwargs):
        if ("betas" in kwargs) and ("gammas" in kwargs):
            b = torch.as_tensor(kwargs["betas"], dtype=torch.float64).reshape(-1)
            c = torch.as_tensor(kwargs["gammas"], dtype=torch.float64).reshape(-1)
            self.param_history_tensor[0] = torch.stack([b, c], dim=1).to(self.param_history_tensor.device)
        optimizer = kwargs.get("optimizer", self.optimizer_info)
        max_iter = kwargs.get("max_iter", self.max_iter)
        h0 = self.param_history_tensor[0].clone()
        self.__init__(self.circuit, optimizer, h0[:, 0], h0[:, 1], max_iter)
