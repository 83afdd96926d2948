"""Sensitivity checks for the adjoint -- TEST INFRASTRUCTURE.

Given a model and a recorded step sequence (``oracle.solve_recorded``: the
kind and size of every state-changing step and the step index of every
sample), this module replays the same sequence with other rate constants
(backward-Euler steps solved to convergence, RKF45 steps with the Fehlberg
stages of kernels.cuh:68-182 and the 4th-order combination kept on
acceptance), and differentiates the misfit

    L(log k) = sum over samples and sampled species of (y - target)^2

by central finite differences and by FP64 forward (tangent-linear)
sensitivities.  Dense numpy linear algebra; sizes up to a few hundred
species.
"""
from __future__ import annotations

import numpy as np

A_RK = np.array([
    [0, 0, 0, 0, 0],
    [1 / 4, 0, 0, 0, 0],
    [3 / 32, 9 / 32, 0, 0, 0],
    [1932 / 2197, -7200 / 2197, 7296 / 2197, 0, 0],
    [439 / 216, -8, 3680 / 513, -845 / 4104, 0],
])
B_RK = np.array([25 / 216, 0, 1408 / 2565, 2197 / 4104, -1 / 5])


class DenseNet:
    """f(y) = S prop(y), prop_j = k_j prod_s y_s^A_js, with exact derivatives."""

    def __init__(self, model):
        self.A = np.asarray(model.left, np.float64)            # R x N
        self.S = (np.asarray(model.right) - np.asarray(model.left)).T.astype(np.float64)
        self.R, self.N = self.A.shape
        self.react = [np.nonzero(self.A[j])[0] for j in range(self.R)]

    def mono(self, y):
        out = np.ones(self.R)
        for j, rs in enumerate(self.react):
            for s in rs:
                out[j] *= y[s] ** self.A[j, s]
        return out

    def f(self, k, y):
        return self.S @ (k * self.mono(y))

    def dprop(self, k, y):
        D = np.zeros((self.R, self.N))
        for j, rs in enumerate(self.react):
            for g in rs:
                a = self.A[j, g]
                d = k[j] * a * y[g] ** (a - 1)
                for o in rs:
                    if o != g:
                        d *= y[o] ** self.A[j, o]
                D[j, g] = d
        return D

    def J(self, k, y):
        return self.S @ self.dprop(k, y)

    def f_logk(self, k, y):
        return self.S * (k * self.mono(y))[None, :]            # N x R


def _be_solve(net, k, y, h, tol=1e-14, iters=60):
    z = y.copy()
    I = np.eye(net.N)
    for _ in range(iters):
        g = z - y - h * net.f(k, z)
        dz = np.linalg.solve(I - h * net.J(k, z), g)
        z = z - dz
        if np.max(np.abs(dz)) <= tol * (1.0 + np.max(np.abs(z))):
            break
    return z


def _rk_stages(net, k, y, h):
    Y, K = [], []
    for i in range(5):
        Yi = y + sum(A_RK[i, j] * K[j] for j in range(i)) if i else y.copy()
        Y.append(Yi)
        K.append(h * net.f(k, Yi))
    return Y, K


def replay(model, k, kinds, dts, samp, net=None):
    """Trajectory at the samples for rate constants k along a frozen step
    sequence (no fed species)."""
    assert model.feed is None
    net = net or DenseNet(model)
    cs = model.sampled()
    y = np.asarray(model.x0, np.float64).copy()
    out = np.zeros((len(samp), cs.size))
    ip = 0
    while ip < len(samp) and samp[ip] == 0:
        out[ip] = y[cs]
        ip += 1
    for n, (kd, h) in enumerate(zip(kinds, dts)):
        if kd == 0:
            Y, K = _rk_stages(net, k, y, h)
            y = y + sum(B_RK[i] * K[i] for i in range(5))
        elif kd == 1:
            y = _be_solve(net, k, y, h)
        while ip < len(samp) and samp[ip] == n + 1:
            out[ip] = y[cs]
            ip += 1
    return out


def loss(model, logk, target, kinds, dts, samp, net=None):
    out = replay(model, np.exp(logk), kinds, dts, samp, net)
    return float(np.sum((out - target) ** 2))


def fd_gradient(model, logk, target, kinds, dts, samp, idx, h=1e-6):
    """Central differences of the replayed loss in the log k components idx."""
    net = DenseNet(model)
    g = []
    for j in idx:
        e = np.zeros_like(logk)
        e[j] = h
        g.append((loss(model, logk + e, target, kinds, dts, samp, net)
                  - loss(model, logk - e, target, kinds, dts, samp, net)) / (2 * h))
    return np.array(g)


def tlm_directional(model, logk, target, kinds, dts, samp, v):
    """dL/dlog k . v by FP64 forward sensitivities along the frozen sequence."""
    net = DenseNet(model)
    k = np.exp(logk)
    cs = model.sampled()
    y = np.asarray(model.x0, np.float64).copy()
    yd = np.zeros_like(y)
    I = np.eye(net.N)
    dL = 0.0
    ip = 0

    def sample(y, yd):
        nonlocal ip, dL
        while ip < len(samp) and samp_now(ip):
            dL += float(np.sum(2 * (y[cs] - target[ip]) * yd[cs]))
            ip += 1

    step = [0]
    samp_now = lambda i: samp[i] == step[0]  # noqa: E731
    sample(y, yd)
    for n, (kd, h) in enumerate(zip(kinds, dts)):
        if kd == 0:
            Y, K = _rk_stages(net, k, y, h)
            Kd = []
            for i in range(5):
                Yd = yd + sum(A_RK[i, j] * Kd[j] for j in range(i)) if i else yd
                Kd.append(h * (net.J(k, Y[i]) @ Yd + net.f_logk(k, Y[i]) @ v))
            y = y + sum(B_RK[i] * K[i] for i in range(5))
            yd = yd + sum(B_RK[i] * Kd[i] for i in range(5))
        elif kd == 1:
            y = _be_solve(net, k, y, h)
            yd = np.linalg.solve(I - h * net.J(k, y), yd + h * (net.f_logk(k, y) @ v))
        step[0] = n + 1
        sample(y, yd)
    return dL
