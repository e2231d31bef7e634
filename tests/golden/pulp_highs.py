"""A stand-in for the part of the PuLP modelling package that the reference's ILP partitioner
(squander/partitioning/ilp.py) uses, solving with SciPy's HiGHS MILP (scipy.optimize.milp) in
place of CBC.  Test infrastructure only: make_partition_ilp_golden.py installs it as `pulp`
so that the reference's own partitioner runs here (PuLP, CBC and Gurobi are not in this image).

Provided: LpProblem (`+=` of constraints, setObjective, solve), LpVariable (and .dicts),
lpSum, value, LpMinimize, LpStatus, PULP_CBC_CMD, and GUROBI (raises, so the reference's
CBC path is taken).  Linear expressions support +, -, * by numbers and the comparisons
<=, >=, == that make constraints.  Integer variables are reported rounded to integers, as
CBC's solution files report them.  The solver runs with a zero relative MIP gap, so a
reported optimum is proven optimal."""
import itertools

import numpy as np
from scipy.optimize import Bounds, LinearConstraint, milp
from scipy.sparse import coo_matrix

LpMinimize = 1
LpMaximize = -1
LpStatus = {0: "Not Solved", 1: "Optimal", -1: "Infeasible", -2: "Unbounded", -3: "Undefined"}

_ids = itertools.count()


class LpAffineExpression:
    def __init__(self, terms=None, constant=0.0):
        self.terms = dict(terms or {})  # variable id -> (variable, coefficient)
        self.constant = float(constant)

    @staticmethod
    def of(x):
        if isinstance(x, LpAffineExpression):
            return x
        if isinstance(x, LpVariable):
            return LpAffineExpression({x.id: (x, 1.0)})
        return LpAffineExpression(constant=float(x))

    def _combine(self, other, sign):
        o = LpAffineExpression.of(other)
        terms = dict(self.terms)
        for k, (v, c) in o.terms.items():
            terms[k] = (v, terms[k][1] + sign * c) if k in terms else (v, sign * c)
        return LpAffineExpression(terms, self.constant + sign * o.constant)

    def __add__(self, other):
        return self._combine(other, 1.0)

    __radd__ = __add__

    def __sub__(self, other):
        return self._combine(other, -1.0)

    def __rsub__(self, other):
        return LpAffineExpression.of(other)._combine(self, -1.0)

    def __neg__(self):
        return self * -1.0

    def __mul__(self, k):
        if isinstance(k, (LpAffineExpression, LpVariable)):
            raise TypeError("non-linear product")
        k = float(k)
        return LpAffineExpression({i: (v, c * k) for i, (v, c) in self.terms.items()}, self.constant * k)

    __rmul__ = __mul__

    def __le__(self, other):
        return LpConstraint(self - other, "<=")

    def __ge__(self, other):
        return LpConstraint(self - other, ">=")

    def __eq__(self, other):
        return LpConstraint(self - other, "==")

    __hash__ = object.__hash__

    def value(self):
        return self.constant + sum(c * v.varValue for v, c in self.terms.values())


class LpVariable(LpAffineExpression):
    def __init__(self, name, lowBound=None, upBound=None, cat="Continuous"):
        self.name = str(name)
        self.id = next(_ids)
        self.cat = cat
        if cat == "Binary":
            lowBound, upBound = 0, 1
        self.lowBound = lowBound
        self.upBound = upBound
        self.varValue = None
        super().__init__({self.id: (self, 1.0)}, 0.0)

    @classmethod
    def dicts(cls, name, indices, lowBound=None, upBound=None, cat="Continuous"):
        return {i: cls("%s_%s" % (name, i), lowBound, upBound, cat) for i in indices}

    def value(self):
        return self.varValue

    __hash__ = object.__hash__


class LpConstraint:
    def __init__(self, expr, sense):
        self.expr = expr
        self.sense = sense


def lpSum(items):
    out = LpAffineExpression()
    for x in items:
        out = out + x
    return out


def value(x):
    if isinstance(x, LpAffineExpression):
        return x.value()
    return x


class PULP_CBC_CMD:
    def __init__(self, msg=False, **kwargs):
        pass


class GUROBI:
    def __init__(self, *args, **kwargs):
        raise RuntimeError("Gurobi is not available")


class LpProblem:
    last_objective = None

    def __init__(self, name="NoName", sense=LpMinimize):
        self.name = name
        self.sense = sense
        self.objective = LpAffineExpression()
        self.constraints = []
        self.status = 0

    def __iadd__(self, other):
        if isinstance(other, LpConstraint):
            self.constraints.append(other)
        elif isinstance(other, bool):
            if not other:
                raise ValueError("infeasible constant constraint")
        else:
            self.objective = LpAffineExpression.of(other)
        return self

    def setObjective(self, expr):
        self.objective = LpAffineExpression.of(expr)

    def _variables(self):
        seen = {}
        for e in [self.objective] + [c.expr for c in self.constraints]:
            for k, (v, _) in e.terms.items():
                seen.setdefault(k, v)
        return [seen[k] for k in sorted(seen)]

    def solve(self, solver=None, **kwargs):
        variables = self._variables()
        col = {v.id: j for j, v in enumerate(variables)}
        n = len(variables)
        if n == 0:
            self.status = 1
            LpProblem.last_objective = self.objective.value()
            return self.status
        c = np.zeros(n)
        for k, (v, coef) in self.objective.terms.items():
            c[col[k]] += coef
        if self.sense == LpMaximize:
            c = -c
        rows, cols, vals, lb, ub = [], [], [], [], []
        for r, con in enumerate(self.constraints):
            for k, (v, coef) in con.expr.terms.items():
                rows.append(r)
                cols.append(col[k])
                vals.append(coef)
            rhs = -con.expr.constant
            lb.append(rhs if con.sense in (">=", "==") else -np.inf)
            ub.append(rhs if con.sense in ("<=", "==") else np.inf)
        integrality = np.array([0 if v.cat == "Continuous" else 1 for v in variables])
        lo = np.array([-np.inf if v.lowBound is None else v.lowBound for v in variables], dtype=float)
        hi = np.array([np.inf if v.upBound is None else v.upBound for v in variables], dtype=float)
        cons = []
        if self.constraints:
            A = coo_matrix((vals, (rows, cols)), shape=(len(self.constraints), n)).tocsr()
            cons = [LinearConstraint(A, np.array(lb), np.array(ub))]
        res = milp(c, integrality=integrality, bounds=Bounds(lo, hi), constraints=cons,
                   options={"mip_rel_gap": 0.0})
        if res.x is None:
            self.status = -1
            raise RuntimeError("MILP not solved: %s" % res.message)
        self.status = 1
        for j, v in enumerate(variables):
            v.varValue = float(round(res.x[j])) if integrality[j] else float(res.x[j])
        LpProblem.last_objective = self.objective.value()
        return self.status
