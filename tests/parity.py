"""Comparison helpers shared by the parity tests.

Tolerances (FP32, one step, library vs the reference's FP32 step):
  counts       bit-exact
  acceleration |a - a_ref| <= 1e-5 * m_i per component, m_i = the FP64
               oracle's |scale| * sum_j |F_j| (rep e^{-k r^2} + att r): the
               size of the quantities whose rounded combination is the force
               (each term is a repulsion-minus-attraction difference that
               cancels near r ~ 0.37, and the terms are summed).  Summation
               order (cell order against index order) and few-ulp rsqrt/exp
               approximations move the result by a few ulp of those
               quantities, never of the (possibly cancelled) result.
  velocity     |v - v_ref| <= 1e-5 * (|v_ref| + dt * m_i)
  position     minimum-image |p - p_ref| <= 1e-5 * |p_ref| + 2 ulp(extent) + dt * (velocity
               tolerance): the position is p + v dt, so the velocity's allowed error
               carries over (it matters where thousands of large terms nearly cancel)
"""

from __future__ import annotations

import numpy as np

REL = 1e-5


def min_image(d: np.ndarray, extent: float) -> np.ndarray:
    return d - extent * np.round(d / extent)


def acc_error(acc, acc_ref, mag) -> float:
    """Largest per-component error in units of the term magnitude."""
    diff = np.abs(np.asarray(acc, np.float64) - np.asarray(acc_ref, np.float64))
    scale = np.maximum(np.asarray(mag, np.float64), 1e-30)[:, None]
    return float((diff / scale).max()) if len(diff) else 0.0


def check_step(rec, ref_pos, ref_vel, ref_acc, mag, dt, extent, label=""):
    """Assert one step's library output matches the FP32 reference within the stated tolerances."""
    acc = np.asarray(rec["acc"], np.float64)
    vel = np.asarray(rec["vel"], np.float64)
    pos = np.asarray(rec["pos"], np.float64)
    e_acc = acc_error(acc, ref_acc, mag)
    assert e_acc <= REL, f"{label} acceleration error {e_acc:.3e} x term size"
    vtol = REL * (np.abs(ref_vel) + dt * np.asarray(mag)[:, None]) + 1e-30
    e_vel = (np.abs(vel - ref_vel) / vtol).max() if len(vel) else 0.0
    assert e_vel <= 1.0, f"{label} velocity error {e_vel:.3e} of tolerance"
    ptol = REL * np.abs(np.asarray(ref_pos, np.float64)) + 2 * np.spacing(np.float32(extent)) + dt * vtol
    dpos = np.abs(min_image(pos - ref_pos, extent))
    e_pos = (dpos / ptol).max() if len(pos) else 0.0
    assert e_pos <= 1.0, f"{label} position error {e_pos:.3e} of tolerance"
    return {"acc": e_acc, "vel": float(e_vel), "pos": float(e_pos)}


def edge_set(edges) -> set:
    return {(int(a), int(b)) for a, b in np.asarray(edges).reshape(-1, 2)}
