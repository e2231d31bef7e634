"""Host-side optimisers driving single decompositions through the GPU cost/gradient.

``bfgs_powell`` restates SQUANDER's BFGS with Powell's conjugate-direction (Z-matrix)
update and its line search:
  src-cpp/common/BFGS_Powell.cpp:70-192 (Optimize), :202-396 (BFGS_iteration),
  :407-446 (get_search_direction);
  src-cpp/common/grad_descend.cpp:127-273 (line_search), :399-425 (maximal step).
The cost-and-gradient callback is the engine's adjoint kernel.
"""
import math

import numpy as np

NUM_PRECISION = 1.42e-14  # grad_descend.cpp:37


def _bfgs_update(Z, ztg, x, g, x0, g0, norm_Z):
    n = x.size
    delta = x - x0
    gamma = g - g0
    norm_delta = float(delta @ delta)
    tmp = float(g0 @ delta)
    dtg = float(gamma @ delta)
    if dtg < abs(tmp) * 0.1:
        return norm_Z
    dtg = max(NUM_PRECISION, dtg)
    # Givens rotations confining Z^T g to the first column (BFGS_Powell.cpp:249-278)
    for col in range(n - 1, 0, -1):
        if ztg[col] == 0.0:
            continue
        cm = col - 1
        a = math.sqrt(ztg[cm] * ztg[cm] + ztg[col] * ztg[col])
        cv, sv = ztg[cm] / a, ztg[col] / a
        ztg[cm] = a
        zc = Z[:, cm].copy()
        zn = Z[:, col].copy()
        Z[:, col] = cv * zn - sv * zc
        Z[:, cm] = cv * zc + sv * zn
    if norm_Z < 0.0:
        norm_Z = norm_delta / dtg
    else:
        t = math.sqrt(norm_Z * norm_delta / dtg)
        norm_Z = min(norm_Z, t)
        norm_Z = max(norm_Z, t * 0.1)
    t = math.sqrt(dtg)
    Z[:, 0] = np.where(np.abs(delta) > NUM_PRECISION, delta / t, 0.0)
    gTz = (gamma @ Z[:, 1:]) / dtg
    Z[:, 1:] -= np.outer(delta, gTz)
    nz = np.einsum("ij,ij->j", Z[:, 1:], Z[:, 1:])
    scale = np.where((nz < norm_Z) & (nz > NUM_PRECISION), np.sqrt(norm_Z / np.where(nz > 0, nz, 1.0)), 1.0)
    Z[:, 1:] *= scale
    return norm_Z


def bfgs_powell(fg, x, max_calls=10000):
    """Minimise fg (x -> (f, grad)) from x (modified in place).  Returns (f, calls)."""
    n = x.size
    Z = np.eye(n)
    norm_Z = -1.0
    calls = 1
    f, g = fg(x)
    fprev = abs(f + f + 1.0)
    while True:
        ztg = Z.T @ g
        d = -(Z @ ztg)
        dg = float(d @ g)
        max_step = 0.0
        if dg < 0.0:
            big = np.abs(d) >= 1e-5
            if big.any():
                max_step = float(np.min(np.abs(2 * math.pi / d[big])))
        if float(g @ g) <= 1e-19 * 1e-19 or dg >= 0.0 or f >= fprev:
            break
        fprev = f
        if calls >= max_calls:
            break
        x0 = x.copy()
        g0 = g.copy()
        gbest = g.copy()
        step = min(1.0, max_step)
        f_low = f_high = f
        s_high, s_low, s_best, f_best = max_step, 0.0, 0.0, f
        dg_best = abs(dg)
        dg_high = 0.0
        for it in range(50):
            x[:] = x0 + step * d
            f, g = fg(x)
            calls += 1
            dgc = float(d @ g)
            if f < f_best or abs(dgc) < dg_best:
                s_best, f_best, dg_best = step, f, abs(dgc)
                gbest = g.copy()
            if calls == max_calls:
                break
            if f < f_low + step * 0.1 * dg:
                if dgc >= dg * 0.7:
                    break
                s_low, f_low = step, f
            else:
                s_high, f_high, dg_high = step, f, dgc
            if it == 0 or s_low > 0.0:
                # IEEE semantics as in the C++ reference (a zero bracket gives inf/nan and
                # std::max(0.1, nan) == 0.1)
                with np.errstate(all="ignore"):
                    dlf = np.float64(f_high - f_low) / np.float64(s_high - s_low) * 2.0 - dg_high
                    scale = -dlf * 0.5 / np.float64(dg_high - dlf)
                scale = float(scale) if scale > 0.1 else 0.1
                step = s_low + scale * (s_high - s_low)
            else:
                step *= 0.1
                if step < NUM_PRECISION:
                    break
        if step != s_best:
            step, f, g = s_best, f_best, gbest
            x[:] = x0 + step * d
        if step == 0.0:
            break
        norm_Z = _bfgs_update(Z, ztg, x, g, x0, g0, norm_Z)
    return f, calls


def adam(fg, x, max_calls=10000, eta=0.01, beta1=0.9, beta2=0.999, eps=1e-8, tol=None):
    """Plain Adam on fg; stops at max_calls or when f < tol.  Returns (f_best, calls)."""
    m = np.zeros_like(x)
    v = np.zeros_like(x)
    best_f, best_x = math.inf, x.copy()
    for t in range(1, max_calls + 1):
        f, g = fg(x)
        if f < best_f:
            best_f, best_x = f, x.copy()
        if tol is not None and f < tol:
            break
        m = beta1 * m + (1 - beta1) * g
        v = beta2 * v + (1 - beta2) * g * g
        mh = m / (1 - beta1 ** t)
        vh = v / (1 - beta2 ** t)
        x -= eta * mh / (np.sqrt(vh) + eps)
    x[:] = best_x
    return best_f, t
