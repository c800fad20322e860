"""Analytic reference solutions shared by the CPU and GPU tests."""
import numpy as np


def shapiro_exact(N, t, nu):
    # ShapiroExactSolution, solver.c:1654-1702 (A = 2, K = L = M = 2), with the
    # w component's sin(Mz) of Shapiro's solution (defect D13: solver.c:1686 has cos)
    A, K, L, M = 2.0, 2.0, 2.0, 2.0
    lam = np.sqrt(K * K + L * L + M * M)
    x = np.arange(N) * 2 * np.pi / N
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    d = np.exp(-lam ** 2 * t * nu)
    u = -A / (K * K + L * L) * (lam * L * np.cos(K * X) * np.sin(L * Y) * np.sin(M * Z) + M * K * np.sin(K * X) * np.cos(L * Y) * np.cos(M * Z)) * d
    v = A / (K * K + L * L) * (lam * K * np.sin(K * X) * np.cos(L * Y) * np.sin(M * Z) - M * L * np.cos(K * X) * np.sin(L * Y) * np.cos(M * Z)) * d
    w = A * np.cos(K * X) * np.cos(L * Y) * np.sin(M * Z) * d
    return np.stack([u, v, w], -1)
