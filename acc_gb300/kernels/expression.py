"""E(Q) and S(Q) expressions of the E_Q kernel, compiled to postfix programs.

The reference turns the expression strings into device functions by
exec-ing "def E_Q_func(Q): return <expr>" with the names of Python's math
module in scope, after replacing "^" by "**" (acc/kernels/E_Q.py:16-34).
Here the host parses the same strings with `ast` and emits a postfix
program of {opcode, argument} pairs (MCV_EXPR_* of the C header) that the
device kernels and the oracle evaluate on a stack of MCV_EXPR_STACK values.

Accepted: numbers, Q, pi, e, unary +/-, + - * / // % **, and the calls
exp log(x[, base]) log10 sqrt sin cos tan asin acos atan atan2 sinh cosh
tanh asinh acosh atanh erf erfc fabs abs floor ceil pow min max.  Constant
subexpressions are folded in float64 on the host; x**n with an integer
constant n is POWI (binary powering).  Anything else (comparisons,
conditionals, other names) raises ValueError here rather than failing on
the device.
"""

import ast
import math

import numpy as np

from .. import _native as nat

CONST, Q_, ADD, SUB, MUL, DIV, POW, NEG, POWI, ATAN2, MIN, MAX, MOD = (
    1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13)
UNARY = {
    "exp": 16, "log": 17, "log10": 18, "sqrt": 19, "sin": 20, "cos": 21,
    "tan": 22, "asin": 23, "acos": 24, "atan": 25, "sinh": 26, "cosh": 27,
    "tanh": 28, "asinh": 29, "acosh": 30, "atanh": 31, "erf": 32,
    "erfc": 33, "fabs": 34, "abs": 34, "floor": 35, "ceil": 36,
}
BINARY_CALLS = {"atan2": ATAN2, "pow": POW, "min": MIN, "max": MAX}
BINOPS = {ast.Add: ADD, ast.Sub: SUB, ast.Mult: MUL, ast.Div: DIV,
          ast.Pow: POW, ast.Mod: MOD}
NAMES = {"pi": math.pi, "e": math.e}
STACK = nat.MCV_EXPR_STACK
MAX_OPS = nat.MCV_EXPR_MAX_OPS

_PY = {ADD: lambda a, b: a + b, SUB: lambda a, b: a - b,
       MUL: lambda a, b: a * b, DIV: lambda a, b: a / b,
       POW: lambda a, b: math.pow(a, b), ATAN2: math.atan2,
       MIN: min, MAX: max, MOD: lambda a, b: a % b}


def _const(node):
    return node[0] == "c"


def _fold(op, *args):
    """Fold an operation of constant operands; None when Python raises
    (division by zero, domain errors): the program then computes it."""
    vals = [a[1] for a in args]
    try:
        if op in _PY:
            return float(_PY[op](*vals))
        if op == NEG:
            return -vals[0]
        name = {v: k for k, v in UNARY.items() if k != "abs"}[op]
        return float(getattr(math, name)(vals[0]))
    except (ArithmeticError, ValueError, OverflowError):
        return None


def _node(op, *args):
    if args and all(_const(a) for a in args):
        v = _fold(op, *args)
        if v is not None:
            return ("c", v)
    return ("op", op, args)


def _build(tree):
    """ast -> nested ("c", value) | ("q",) | ("op", code, args) | ("powi", n, x)"""
    if isinstance(tree, ast.Expression):
        return _build(tree.body)
    if isinstance(tree, ast.Constant) and isinstance(tree.value, (int, float)) \
            and not isinstance(tree.value, bool):
        return ("c", float(tree.value))
    if isinstance(tree, ast.Name):
        if tree.id == "Q":
            return ("q",)
        if tree.id in NAMES:
            return ("c", NAMES[tree.id])
        raise ValueError("unknown name %r in expression" % tree.id)
    if isinstance(tree, ast.UnaryOp):
        x = _build(tree.operand)
        if isinstance(tree.op, ast.UAdd):
            return x
        if isinstance(tree.op, ast.USub):
            return _node(NEG, x)
        raise ValueError("unsupported unary operator")
    if isinstance(tree, ast.BinOp):
        a, b = _build(tree.left), _build(tree.right)
        if isinstance(tree.op, ast.FloorDiv):
            return _node(UNARY["floor"], _node(DIV, a, b))
        if isinstance(tree.op, ast.Pow) and _const(b) and not _const(a) \
                and float(b[1]).is_integer() and abs(b[1]) <= 64:
            return ("powi", int(b[1]), a)
        op = BINOPS.get(type(tree.op))
        if op is None:
            raise ValueError("unsupported operator %s" % type(tree.op).__name__)
        return _node(op, a, b)
    if isinstance(tree, ast.Call):
        if not isinstance(tree.func, ast.Name) or tree.keywords:
            raise ValueError("unsupported call")
        name, args = tree.func.id, [_build(a) for a in tree.args]
        if name == "log" and len(args) == 2:
            return _node(DIV, _node(UNARY["log"], args[0]),
                         _node(UNARY["log"], args[1]))
        if name in UNARY and len(args) == 1:
            return _node(UNARY[name], args[0])
        if name in BINARY_CALLS and len(args) == 2:
            if name == "pow" and _const(args[1]) and not _const(args[0]) \
                    and float(args[1][1]).is_integer() and abs(args[1][1]) <= 64:
                return ("powi", int(args[1][1]), args[0])
            return _node(BINARY_CALLS[name], *args)
        raise ValueError("unsupported function %s/%d" % (name, len(args)))
    raise ValueError("unsupported expression element %s" % type(tree).__name__)


def _emit(node, out):
    """Postfix emission; returns the stack depth the subtree needs."""
    kind = node[0]
    if kind == "c":
        out.append((CONST, node[1]))
        return 1
    if kind == "q":
        out.append((Q_, 0.0))
        return 1
    if kind == "powi":
        d = _emit(node[2], out)
        out.append((POWI, float(node[1])))
        return d
    _, op, args = node
    if len(args) == 1:
        d = _emit(args[0], out)
        out.append((op, 0.0))
        return d
    d0 = _emit(args[0], out)
    d1 = _emit(args[1], out)
    out.append((op, 0.0))
    return max(d0, d1 + 1)


def compile_expression(text):
    """The expression string (in Q) -> float64 array (nops, 2) of
    {opcode, argument}.  "^" means "**", as in the reference."""
    text = str(text).replace("^", "**")
    try:
        tree = ast.parse(text.strip(), mode="eval")
    except SyntaxError as exc:
        raise ValueError("cannot parse expression %r: %s" % (text, exc))
    prog = []
    depth = _emit(_build(tree), prog)
    if depth > STACK:
        raise ValueError("expression %r needs a stack of %d (at most %d)"
                         % (text, depth, STACK))
    if len(prog) > MAX_OPS:
        raise ValueError("expression %r compiles to %d instructions (at most %d)"
                         % (text, len(prog), MAX_OPS))
    return np.asarray(prog, dtype=np.float64).reshape(-1, 2)


def evaluate(prog, Q):
    """Host evaluation of a compiled program (float64), for checks."""
    st = []
    for op, arg in np.asarray(prog, dtype=np.float64).reshape(-1, 2):
        op = int(op)
        if op == CONST:
            st.append(float(arg))
        elif op == Q_:
            st.append(float(Q))
        elif op == POWI:
            st.append(st.pop() ** int(arg))
        elif op == NEG:
            st.append(-st.pop())
        elif op in _PY:
            b, a = st.pop(), st.pop()
            st.append(float(_PY[op](a, b)))
        else:
            name = {v: k for k, v in UNARY.items() if k != "abs"}[op]
            st.append(float(getattr(math, name)(st.pop())))
    assert len(st) == 1
    return st[0]
