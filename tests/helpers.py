"""Shared comparison helpers for the parity tests."""
import numpy as np


def rowwise_rel(a, b):
    """max over rows of ||a_row - b_row||_inf / max(||b_row||_inf, 1)."""
    a = np.asarray(a, dtype=np.float64).reshape(-1, np.shape(a)[-1])
    b = np.asarray(b, dtype=np.float64).reshape(-1, np.shape(b)[-1])
    num = np.max(np.abs(a - b), axis=1)
    den = np.maximum(np.max(np.abs(b), axis=1), 1.0)
    return float(np.max(num / den)) if num.size else 0.0


def stm_state(x6):
    y = np.zeros(42)
    y[:36] = np.eye(6).ravel()
    y[36:] = x6
    return y
