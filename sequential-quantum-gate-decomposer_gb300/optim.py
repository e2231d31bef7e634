"""Host-side optimisers driving single decompositions through the GPU cost/gradient.

``bfgs_powell`` restates SQUANDER's BFGS with Powell's conjugate-direction (Z-matrix)
update and its line search:
  src-cpp/common/BFGS_Powell.cpp:70-192 (Optimize), :202-396 (BFGS_iteration),
  :407-446 (get_search_direction);
  src-cpp/common/grad_descend.cpp:127-273 (line_search), :399-425 (maximal step).
``adam_squander`` restates SQUANDER's ADAM engine (optimization_engines/ADAM.cpp:44-330 with
common/Adam.cpp), the optimizer N_Qubit_Decomposition_custom picks above five qubits.
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


_MASK = (1 << 64) - 1


class SplitMix64:
    """Seeded splitmix64 stream (Steele, Lea and Flood 2014), the random source of every
    decomposition driver of this package; u01() = top 53 bits / 2^53."""

    def __init__(self, seed):
        self.s = int(seed) & _MASK

    def next(self):
        self.s = (self.s + 0x9E3779B97F4A7C15) & _MASK
        z = self.s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _MASK
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _MASK
        return z ^ (z >> 31)

    def u01(self):
        return (self.next() >> 11) * (1.0 / 9007199254740992.0)


class AdamState:
    """SQUANDER's Adam (src-cpp/common/Adam.cpp): beta1 0.68, beta2 0.8, epsilon 1e-4
    (:31-40), moments, the 100-value cost window and the 20-step decreasing test of its
    local-minimum detector (reset :70-100, update :138-270).  The bias-correction powers
    advance once per parameter, in parameter order, as the reference's parameter loop does."""

    def __init__(self, P, eta):
        self.beta1, self.beta2, self.eps, self.eta = 0.68, 0.8, 1e-4, eta
        self.P = P
        self.reset()

    def reset(self):
        self.mom = np.zeros(self.P)
        self.var = np.zeros(self.P)
        self.beta1_t = 1.0
        self.beta2_t = 1.0
        self.f0_vec = np.zeros(100)
        self.f0_mean = 0.0
        self.f0_idx = 0
        self.dec_vec = [-1] * 20
        self.dec_idx = 0
        self.dec_test = -1.0
        self.f0_prev = np.finfo(np.float64).max

    def update(self, x, g, f0):
        """One Adam step of x in place; returns 1 when the local-minimum test fires."""
        self.f0_mean = self.f0_mean + (f0 - self.f0_vec[self.f0_idx]) / 100
        self.f0_vec[self.f0_idx] = f0
        self.f0_idx = (self.f0_idx + 1) % 100
        var_f0 = 0.0
        for v in self.f0_vec:
            var_f0 = var_f0 + (v - self.f0_mean) * (v - self.f0_mean)
        var_f0 = math.sqrt(var_f0) / 100
        if f0 < self.f0_prev:
            if self.dec_vec[self.dec_idx] != 1:
                self.dec_test = self.dec_test + 2.0 / 20
            self.dec_vec[self.dec_idx] = 1
        else:
            if self.dec_vec[self.dec_idx] == 1:
                self.dec_test = self.dec_test - 2.0 / 20
            self.dec_vec[self.dec_idx] = -1
        self.dec_idx = (self.dec_idx + 1) % 20
        self.f0_prev = f0
        grad_var = 0.0
        for v in self.var:
            grad_var += v
        eps = self.eps / 100 if (grad_var < self.eps and self.dec_test > 0.7) else self.eps
        b1, b2 = self.beta1, self.beta2
        self.mom = b1 * self.mom + (1 - b1) * g
        self.var = b2 * self.var + (1 - b2) * g * g
        # beta_t advanced per parameter: beta1_t * beta1^(i + 1) by repeated multiplication
        p1 = np.empty(self.P)
        p2 = np.empty(self.P)
        t1, t2 = self.beta1_t, self.beta2_t
        for i in range(self.P):
            t1 = t1 * b1
            t2 = t2 * b2
            p1[i] = t1
            p2[i] = t2
        self.beta1_t, self.beta2_t = t1, t2
        mh = self.mom / (1 - p1)
        vh = self.var / (1 - p2)
        x -= self.eta * mh / (np.sqrt(vh) + eps)
        if abs(self.f0_mean - f0) < 1e-6 and self.dec_test <= 0.7 and var_f0 / self.f0_mean < 1e-6:
            return 1
        return 0


def adam_squander(fg, x, max_iters=100000, tol=1e-8, eta=1e-3, adaptive_eta=True, random_shift_count_max=100,
                  randomization_threshold=2500000, seed=0, current_minimum=None, info=None):
    """SQUANDER's ADAM decomposition engine (Optimization_Interface::
    solve_layer_optimization_problem_ADAM, src-cpp/optimization_engines/ADAM.cpp:44-330):
    Adam steps with the adaptive learning rate, the hold/sub-iteration bookkeeping and,
    when Adam reports a local minimum, a randomisation of 30% of the parameters around the
    best point by U(-2 pi, 2 pi) * sqrt(f) (randomize_parameters,
    decomposition/Optimization_Interface.cpp:576-607), at most random_shift_count_max times.
    x is replaced by the best point.  Returns (minimum cost, evaluations); info (a dict, if
    given) receives the number of randomisations under "shifts"."""
    P = x.size
    rng = SplitMix64(seed)
    opt = AdamState(P, eta)
    xt = x.copy()
    best = x.copy()
    big = np.finfo(np.float64).max
    cur_min = big if current_minimum is None else current_minimum
    hold = cur_min
    sub_iter, shifts, status, n = 0, 0, 0, 0
    for _ in range(max_iters):
        f0, g = fg(xt)
        n += 1
        if sub_iter == 1:
            hold = f0
            if adaptive_eta:
                opt.eta = opt.eta if opt.eta > 1e-3 else 1e-3
        if hold * 0.95 > f0 or (hold * 0.97 > f0 and f0 < 1e-3) or (hold * 0.99 > f0 and f0 < 1e-4):
            sub_iter = 0
            hold = f0
        if cur_min > f0:
            cur_min = f0
            best[:] = xt
            if adaptive_eta:  # the second clamp overwrites the first, as in the reference
                ne = 1e-3 * f0
                opt.eta = ne if ne > 1e-6 else 1e-6
                opt.eta = ne if ne < 1e-1 else 1e-1
        if f0 < tol or shifts > random_shift_count_max:
            break
        if sub_iter > randomization_threshold or status != 0:
            sub_iter = 0
            shifts += 1
            hold = cur_min
            r = math.sqrt(f0)
            for j in range(P):
                if rng.u01() <= 0.3:
                    xt[j] = best[j] + (-2 * math.pi + 4 * math.pi * rng.u01()) * r * 1.0
                else:
                    xt[j] = best[j]
            opt.reset()
            status = 0
        else:
            status = opt.update(xt, g, f0)
        sub_iter += 1
    x[:] = best
    if info is not None:
        info["shifts"] = shifts
    return cur_min, n
