"""Lowering of general compute() kernels of point-mass programs to CUDA.

The reference prints a C/CUDA kernel for every compute() function: it walks the
function's AST (src/pairs/mapping/funcs.py:39-282) with the keyword set of
src/pairs/mapping/keywords.py, wraps a pair kernel in the Verlet-list loop with the
cutoff test (sim/interaction.py:43-129, 201-292) and a particle kernel in a loop over
the particles that are not fixed (mapping/funcs.py:296-299).  Kernels that match the
LJ / velocity-Verlet templates (kernels.py) run on the hand-tuned kernels; any other
point-mass kernel comes here.  This module translates it into a CUDA kernel with the
same statement and operation order, in FP64, compiled with -fmad=false so that every
operation is rounded as in the reference's generated C.

Supported (the reference DSL for point masses):
  statements    local assignments, augmented assignments, prop[i] (=, +=, -=, *=, /=)
                in particle kernels, if / else, apply(prop, vector) and
                skip_when(condition) in pair kernels (skip_when also in particle
                kernels)
  expressions   + - * / % on scalars and 3-vectors (vector * scalar, vector / scalar),
                unary -, comparisons, and / or / not, x if c else y, constants,
                symbols of compute(symbols=...), prop[i], prop[j] (pair kernels),
                feature[i, j], delta(i, j), squared_distance(i, j), sqrt, select,
                min, max, length, dot, cross, normalized, squared_length, zero_vector
Anything else raises NotImplementedError naming the function and the construct.
"""
import ast
import hashlib
import inspect
import os
import subprocess
import textwrap

from .types import Types

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
GEN_DIR = os.path.join(HERE, "_gen")

REAL, INT, BOOL, VEC = "real", "int", "bool", "vec"
MAX_PROPS = 16
MAX_FEATURES = 8


def prop_kind(ptype):
    if ptype == Types.Vector:
        return VEC
    if ptype in (Types.Double, Types.Float):
        return REAL
    if ptype in (Types.Int32, Types.Int64, Types.UInt64, Types.Boolean):
        return INT
    raise NotImplementedError(f"property type {ptype} is not supported by the generated kernels")


def c_literal(v):
    if isinstance(v, bool):
        return "1" if v else "0"
    if isinstance(v, int):
        return str(v)
    if isinstance(v, float):
        if v != v or v in (float("inf"), float("-inf")):
            raise NotImplementedError("non-finite literals are not supported")
        r = repr(v)
        return r if ("e" in r or "." in r) else r + ".0"
    raise NotImplementedError(f"literal {v!r} is not supported")


class Val:
    """A typed expression: `code` is a C expression (tuple of three for vectors)."""

    def __init__(self, kind, code):
        self.kind = kind
        self.code = code

    def comp(self, d):
        return self.code[d] if self.kind == VEC else self.code


class Layout:
    """Where each property of the program lives in the kernels' argument block."""

    def __init__(self, sim):
        self.props = {}          # name -> (kind, expression of the base pointer)
        self.slots = []          # user property names in slot order
        pos = sim.position_prop.name
        self.position = pos
        for name, prop in sim.properties.items():
            kind = prop_kind(prop.type)
            if name == pos:
                self.props[name] = (VEC, "a.p.pos")
            elif name == "uid":
                self.props[name] = (INT, "a.p.uid")
            elif name == "flags":
                self.props[name] = (INT, "a.p.flags")
            elif name == "shape":
                continue
            elif name in sim.features:
                self.props[name] = (INT, "a.p.type")
            elif name == "linear_velocity" and kind == VEC:
                self.props[name] = (VEC, "a.p.vel")
            elif name == "mass" and kind == REAL:
                self.props[name] = (REAL, "a.p.mass")
            else:
                if len(self.slots) >= MAX_PROPS:
                    raise NotImplementedError(f"more than {MAX_PROPS} user properties")
                ctype = {VEC: "double", REAL: "double", INT: "int32_t"}[kind]
                self.props[name] = (kind, f"(({ctype} *) a.prop[{len(self.slots)}])")
                self.slots.append(name)
        self.features = {}       # feature property name -> (slot, feature name)
        feats = list(sim.feature_properties.items())
        if len(feats) > MAX_FEATURES:
            raise NotImplementedError(f"more than {MAX_FEATURES} feature properties")
        for k, (name, fp) in enumerate(feats):
            self.features[name] = (k, fp.feature)
        self.type_prop = next(iter(sim.features), None)


class Translator(ast.NodeVisitor):
    """One compute() function -> the body of a CUDA kernel."""

    def __init__(self, sim, layout, func, symbols, pair):
        self.sim = sim
        self.L = layout
        self.fname = func.__name__
        self.symbols = dict(symbols)
        self.pair = pair
        self.lines = []
        self.indent = 1
        self.locals = {}         # name -> kind
        self.applied = []        # property names accumulated by apply()
        self.written = set()     # properties stored to
        self.read_j = set()      # properties read at the partner
        self.tmp = 0
        src = textwrap.dedent(inspect.getsource(func))
        fn = next(n for n in ast.parse(src).body if isinstance(n, ast.FunctionDef))
        self.params = [a.arg for a in fn.args.args]
        if len(self.params) != (2 if pair else 1):
            raise NotImplementedError(f"{self.fname}: {len(self.params)} parameters")
        self.fn = fn

    # ---------------------------------------------------------------- helpers
    def fail(self, node, what):
        raise NotImplementedError(f"{self.fname}: {what} is not supported by the generated kernels "
                                  f"(line {getattr(node, 'lineno', '?')})")

    def emit(self, line):
        self.lines.append("    " * self.indent + line)

    def fresh(self):
        self.tmp += 1
        return f"t{self.tmp}"

    def index_of(self, node):
        if isinstance(node, ast.Name) and node.id in self.params:
            return self.params.index(node.id)
        self.fail(node, "an index other than the kernel's parameters")

    def load(self, name, who, node):
        kind, base = self.L.props[name]
        idx = "i" if who == 0 else "j"
        if who == 1:
            self.read_j.add(name)
        if self.pair and name == self.L.position:
            # the partner's position is its listed image (the reference's ghost)
            return Val(VEC, ("xi_x", "xi_y", "xi_z") if who == 0 else ("jx", "jy", "jz"))
        if kind == VEC:
            return Val(VEC, tuple(f"{base}[4 * (size_t) {idx} + {d}]" for d in range(3)))
        return Val(kind, f"{base}[{idx}]")

    # ---------------------------------------------------------------- statements
    def body(self):
        for st in self.fn.body:
            self.stmt(st)

    def stmt(self, node):
        if isinstance(node, ast.Expr):
            if isinstance(node.value, ast.Constant) and isinstance(node.value.value, str):
                return                                  # docstring
            if isinstance(node.value, ast.Call) and isinstance(node.value.func, ast.Name):
                name = node.value.func.id
                if name == "apply":
                    return self.apply(node.value)
                if name == "skip_when":
                    c = self.expr(node.value.args[0])
                    self.emit(f"if({self.truth(c)}) {{ {'continue' if self.pair else 'return'}; }}")
                    return
            self.fail(node, "this expression statement")
        if isinstance(node, ast.Assign):
            if len(node.targets) != 1:
                self.fail(node, "multiple assignment targets")
            return self.assign(node.targets[0], node.value, None, node)
        if isinstance(node, ast.AugAssign):
            return self.assign(node.target, node.value, node.op, node)
        if isinstance(node, ast.If):
            c = self.expr(node.test)
            self.emit(f"if({self.truth(c)}) {{")
            self.indent += 1
            for s in node.body:
                self.stmt(s)
            self.indent -= 1
            if node.orelse:
                self.emit("} else {")
                self.indent += 1
                for s in node.orelse:
                    self.stmt(s)
                self.indent -= 1
            self.emit("}")
            return
        if isinstance(node, ast.Pass):
            return
        self.fail(node, type(node).__name__)

    def assign(self, target, value, op, node):
        rhs = self.expr(value)
        if isinstance(target, ast.Name):
            name = target.id
            if name in self.params or name in self.L.props or name in self.symbols:
                self.fail(node, f"assignment to {name!r}")
            if op is not None:
                if name not in self.locals:
                    self.fail(node, f"augmented assignment to undefined {name!r}")
                rhs = self.binop(Val(self.locals[name], self.local_code(name, self.locals[name])), rhs, op, node)
            kind = REAL if rhs.kind == INT and self.locals.get(name) == REAL else rhs.kind
            if name in self.locals:
                if self.locals[name] != kind:
                    self.fail(node, f"a change of type of {name!r}")
                self.store_local(name, kind, rhs, declare=False)
            else:
                if self.indent > 1:
                    self.fail(node, f"a local ({name!r}) first assigned inside a branch")
                self.locals[name] = kind
                self.store_local(name, kind, rhs, declare=True)
            return
        if isinstance(target, ast.Subscript) and isinstance(target.value, ast.Name):
            pname = target.value.id
            if pname not in self.L.props:
                self.fail(node, f"a store to {pname!r}")
            if self.pair:
                self.fail(node, f"a store to {pname!r} in a pair kernel (use apply)")
            if self.index_of(target.slice) != 0:
                self.fail(node, "a store to another particle")
            cur = self.load(pname, 0, node)
            if op is not None:
                rhs = self.binop(cur, rhs, op, node)
            kind = cur.kind
            if kind == VEC and rhs.kind != VEC:
                self.fail(node, f"a scalar stored to vector {pname!r}")
            if kind != VEC and rhs.kind == VEC:
                self.fail(node, f"a vector stored to scalar {pname!r}")
            self.written.add(pname)
            # evaluate every component before storing any (the right side may read
            # the property itself)
            if kind == VEC:
                names = []
                for d in range(3):
                    t = self.fresh()
                    self.emit(f"const double {t} = {rhs.comp(d)};")
                    names.append(t)
                for d in range(3):
                    self.emit(f"{cur.code[d]} = {names[d]};")
            else:
                ctype = "double" if kind == REAL else "int32_t"
                self.emit(f"{cur.code} = ({ctype}) ({rhs.code});")
            return
        self.fail(node, "this assignment target")

    def local_code(self, name, kind):
        # user locals are prefixed so that they cannot clash with the kernel's own names
        if kind == VEC:
            return tuple(f"v_{name}_{c}" for c in "xyz")
        return f"v_{name}"

    def store_local(self, name, kind, rhs, declare):
        ctype = {REAL: "double", INT: "int", BOOL: "bool"}.get(kind, "double")
        dst = self.local_code(name, kind)
        if kind == VEC:
            vals = [rhs.comp(d) for d in range(3)]
            if declare:
                for d in range(3):
                    self.emit(f"double {dst[d]} = {vals[d]};")
            else:
                ts = []
                for d in range(3):
                    t = self.fresh()
                    self.emit(f"const double {t} = {vals[d]};")
                    ts.append(t)
                for d in range(3):
                    self.emit(f"{dst[d]} = {ts[d]};")
        else:
            self.emit(f"{ctype + ' ' if declare else ''}{dst} = {rhs.code};")

    def apply(self, call):
        if not self.pair:
            self.fail(call, "apply() in a particle kernel")
        if len(call.args) != 2 or not isinstance(call.args[0], ast.Name):
            self.fail(call, "this apply() form")
        pname = call.args[0].id
        if pname not in self.L.props:
            self.fail(call, f"apply() to unknown property {pname!r}")
        kind = self.L.props[pname][0]
        v = self.expr(call.args[1])
        if v.kind != kind and not (kind == REAL and v.kind == INT):
            self.fail(call, f"apply() of a {v.kind} to a {kind} property")
        if pname not in self.applied:
            self.applied.append(pname)
        acc = f"acc_{self.applied.index(pname)}"
        if kind == VEC:
            ts = []
            for d in range(3):
                t = self.fresh()
                self.emit(f"const double {t} = {v.comp(d)};")
                ts.append(t)
            for d, c in enumerate("xyz"):
                self.emit(f"{acc}_{c} = {acc}_{c} + {ts[d]};")
            self.emit(f"if(a.half && code == 0u && !(a.p.flags != nullptr && (a.p.flags[j] & 4))) "
                      f"{{ {self.reaction(pname, ts)} }}")
        else:
            t = self.fresh()
            self.emit(f"const double {t} = {v.code};")
            self.emit(f"{acc} = {acc} + {t};")
            self.emit(f"if(a.half && code == 0u && !(a.p.flags != nullptr && (a.p.flags[j] & 4))) "
                      f"{{ {self.reaction(pname, [t])} }}")
        self.written.add(pname)

    def reaction(self, pname, ts):
        kind, base = self.L.props[pname]
        if kind == VEC:
            return " ".join(f"atomicAdd(&{base}[4 * (size_t) j + {d}], -{ts[d]});" for d in range(3))
        if kind == REAL:
            return f"atomicAdd(&{base}[j], -{ts[0]});"
        raise NotImplementedError(f"{self.fname}: apply() to an integer property")

    # ---------------------------------------------------------------- expressions
    def truth(self, v):
        if v.kind == VEC:
            raise NotImplementedError(f"{self.fname}: a vector used as a condition")
        return v.code

    def expr(self, node):
        if isinstance(node, ast.Constant):
            v = node.value
            if isinstance(v, bool):
                return Val(BOOL, c_literal(v))
            if isinstance(v, int):
                return Val(INT, c_literal(v))
            if isinstance(v, float):
                return Val(REAL, c_literal(v))
            self.fail(node, f"the constant {v!r}")
        if isinstance(node, ast.Name):
            n = node.id
            if n in self.locals:
                return Val(self.locals[n], self.local_code(n, self.locals[n]))
            if n in self.symbols:
                v = self.symbols[n]
                if isinstance(v, (list, tuple)) and len(v) == 3:
                    return Val(VEC, tuple(c_literal(float(x)) for x in v))
                if isinstance(v, bool):
                    return Val(BOOL, c_literal(v))
                return Val(INT if isinstance(v, int) else REAL, c_literal(v))
            self.fail(node, f"the name {n!r}")
        if isinstance(node, ast.BinOp):
            return self.binop(self.expr(node.left), self.expr(node.right), node.op, node)
        if isinstance(node, ast.UnaryOp):
            v = self.expr(node.operand)
            if isinstance(node.op, ast.USub):
                if v.kind == VEC:
                    return Val(VEC, tuple(f"(-{c})" for c in v.code))
                return Val(v.kind, f"(-{v.code})")
            if isinstance(node.op, ast.Not):
                return Val(BOOL, f"(!{self.truth(v)})")
            self.fail(node, "this unary operator")
        if isinstance(node, ast.Compare):
            if len(node.ops) != 1:
                self.fail(node, "a chained comparison")
            ops = {ast.Lt: "<", ast.LtE: "<=", ast.Gt: ">", ast.GtE: ">=", ast.Eq: "==", ast.NotEq: "!="}
            op = ops.get(type(node.ops[0]))
            if op is None:
                self.fail(node, "this comparison")
            a, b = self.expr(node.left), self.expr(node.comparators[0])
            if VEC in (a.kind, b.kind):
                self.fail(node, "a comparison of vectors")
            return Val(BOOL, f"({a.code} {op} {b.code})")
        if isinstance(node, ast.BoolOp):
            op = "&&" if isinstance(node.op, ast.And) else "||"
            vals = [self.truth(self.expr(v)) for v in node.values]
            return Val(BOOL, "(" + f" {op} ".join(vals) + ")")
        if isinstance(node, ast.IfExp):
            return self.select(self.expr(node.test), self.expr(node.body), self.expr(node.orelse), node)
        if isinstance(node, ast.Subscript):
            return self.subscript(node)
        if isinstance(node, ast.Call):
            return self.call(node)
        self.fail(node, type(node).__name__)

    def binop(self, a, b, op, node):
        sym = {ast.Add: "+", ast.Sub: "-", ast.Mult: "*", ast.Div: "/", ast.Mod: "%", ast.BitAnd: "&"}.get(type(op))
        if sym is None:
            self.fail(node, "this operator")
        if a.kind == VEC or b.kind == VEC:
            if sym in ("+", "-"):
                if a.kind != VEC or b.kind != VEC:
                    self.fail(node, "a vector added to a scalar")
                return Val(VEC, tuple(f"({a.code[d]} {sym} {b.code[d]})" for d in range(3)))
            if sym == "*":
                if a.kind == VEC and b.kind == VEC:
                    self.fail(node, "a product of two vectors (use dot or cross)")
                return Val(VEC, tuple(f"({a.comp(d)} * {b.comp(d)})" for d in range(3)))
            if sym == "/":
                if b.kind == VEC:
                    self.fail(node, "a division by a vector")
                return Val(VEC, tuple(f"({a.code[d]} / {b.code})" for d in range(3)))
            self.fail(node, f"the operator {sym} on vectors")
        if sym in ("%", "&"):
            if a.kind != INT or b.kind != INT:
                self.fail(node, f"the operator {sym} on non-integers")
            return Val(INT, f"({a.code} {sym} {b.code})")
        kind = INT if (a.kind == INT and b.kind == INT) else REAL
        return Val(kind, f"({a.code} {sym} {b.code})")

    def select(self, c, x, y, node):
        cond = self.truth(c)
        if x.kind == VEC or y.kind == VEC:
            if x.kind != VEC or y.kind != VEC:
                self.fail(node, "select() of a vector and a scalar")
            return Val(VEC, tuple(f"({cond} ? {x.code[d]} : {y.code[d]})" for d in range(3)))
        kind = INT if (x.kind == INT and y.kind == INT) else (BOOL if x.kind == y.kind == BOOL else REAL)
        return Val(kind, f"({cond} ? {x.code} : {y.code})")

    def subscript(self, node):
        if not isinstance(node.value, ast.Name):
            self.fail(node, "this subscript")
        name = node.value.id
        sl = node.slice
        if name in self.L.features:
            if not isinstance(sl, ast.Tuple) or len(sl.elts) != 2:
                self.fail(node, f"feature property {name!r} with other than [i, j]")
            a, b = (self.index_of(e) for e in sl.elts)
            slot, feature = self.L.features[name]
            ia, ib = ("i" if a == 0 else "j"), ("i" if b == 0 else "j")
            if 1 in (a, b):
                self.read_j.add(feature)
            return Val(REAL, f"a.feat[{slot}][a.p.type[{ia}] * a.feat_n[{slot}] + a.p.type[{ib}]]")
        if name in self.L.props:
            if isinstance(sl, ast.Tuple):
                self.fail(node, f"{name!r} with two indices")
            return self.load(name, self.index_of(sl), node)
        if name in self.locals and self.locals[name] == VEC:
            if isinstance(sl, ast.Constant) and sl.value in (0, 1, 2):
                return Val(REAL, self.local_code(name, VEC)[sl.value])
        self.fail(node, f"the subscript of {name!r}")

    def vec_of(self, v, node, what):
        if v.kind != VEC:
            self.fail(node, f"{what} of a scalar")
        return v

    def call(self, node):
        if not isinstance(node.func, ast.Name):
            self.fail(node, "this call")
        f = node.func.id
        args = node.args
        if f in ("delta", "squared_distance"):
            if not self.pair or len(args) != 2 or [self.index_of(x) for x in args] != [0, 1]:
                self.fail(node, f"{f}() outside a pair kernel's (i, j)")
            return Val(VEC, ("dx", "dy", "dz")) if f == "delta" else Val(REAL, "rsq")
        vals = [self.expr(x) for x in args]
        if f == "sqrt":
            if vals[0].kind == VEC:
                self.fail(node, "sqrt() of a vector")
            return Val(REAL, f"sqrt((double) {vals[0].code})")
        if f == "select":
            return self.select(vals[0], vals[1], vals[2], node)
        if f in ("min", "max"):
            # the reference's Select chain (mapping/keywords.py:67-79)
            acc = vals[0]
            for v in vals[1:]:
                cmp = ast.Lt() if f == "min" else ast.Gt()
                c = Val(BOOL, f"({v.code} {'<' if f == 'min' else '>'} {acc.code})")
                acc = self.select(c, v, acc, node)
            return acc
        if f == "squared_length" or f == "length" or f == "dot":
            a = self.vec_of(vals[0], node, f)
            b = self.vec_of(vals[1], node, f) if f == "dot" else a
            s = f"(((0 + ({a.code[0]} * {b.code[0]})) + ({a.code[1]} * {b.code[1]})) + ({a.code[2]} * {b.code[2]}))"
            return Val(REAL, f"sqrt({s})" if f == "length" else s)
        if f == "cross":
            a, b = (self.vec_of(v, node, f) for v in vals)
            return Val(VEC, (f"(({a.code[1]} * {b.code[2]}) - ({a.code[2]} * {b.code[1]}))",
                             f"(({a.code[2]} * {b.code[0]}) - ({a.code[0]} * {b.code[2]}))",
                             f"(({a.code[0]} * {b.code[1]}) - ({a.code[1]} * {b.code[0]}))"))
        if f == "normalized":
            a = self.vec_of(vals[0], node, f)
            ln = self.fresh()
            self.emit(f"const double {ln} = sqrt(((0 + ({a.code[0]} * {a.code[0]})) + ({a.code[1]} * {a.code[1]})) + "
                      f"({a.code[2]} * {a.code[2]}));")
            inv = self.fresh()
            self.emit(f"const double {inv} = 1.0 / {ln};")
            return Val(VEC, tuple(f"(({ln} > 0.0) ? ({a.code[d]} * {inv}) : 0.0)" for d in range(3)))
        if f == "zero_vector":
            return Val(VEC, ("0.0", "0.0", "0.0"))
        self.fail(node, f"the function {f}()")


# ------------------------------------------------------------------------ kernels

PRELUDE = r'''// Generated from the program's compute() functions by pairs_gb300/codegen.py.
#include <cstdint>
#include <cuda_runtime.h>
#include "pairs_gb300.h"

#define PG_GEN_MAX_PROPS %(max_props)d
#define PG_GEN_MAX_FEATURES %(max_feat)d

struct GenArgs {
    pg_box box;
    pg_particles p;
    pg_neighbor_list list;
    int32_t half;
    int32_t sync_ref;
    int32_t feat_n[PG_GEN_MAX_FEATURES];
    const double *feat[PG_GEN_MAX_FEATURES];
    void *prop[PG_GEN_MAX_PROPS];
};

__device__ __forceinline__ double gen_image(double xj, int s, double len) {
    return s == 0 ? xj : __dadd_rn(xj, s > 0 ? len : -len);
}

__device__ __forceinline__ int gen_shift(uint32_t code, int d) {
    const uint32_t c = (code >> (2 * d)) & 3u;
    return c == 1u ? 1 : (c == 2u ? -1 : 0);
}

__device__ __forceinline__ int gen_image_dims(uint32_t code) {
    return (int) ((code & 3u) != 0u) + (int) (((code >> 2) & 3u) != 0u) + (int) (((code >> 4) & 3u) != 0u);
}
'''

PAIR = r'''
// pair kernel %(name)s: Verlet list of particle i, cutoff %(cutoff)r
extern "C" __global__ void __launch_bounds__(256) k_%(name)s(GenArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= a.p.n) { return; }
    if(a.p.flags != nullptr && (a.p.flags[i] & 4)) { return; }
%(acc_decl)s    const double xi_x = a.p.pos[4 * (size_t) i], xi_y = a.p.pos[4 * (size_t) i + 1], xi_z = a.p.pos[4 * (size_t) i + 2];
    const int cnt = a.list.count[i];
    for(int k = 0; k < cnt; k++) {
        const uint32_t e = (uint32_t) a.list.nbr[(size_t) k * a.list.stride + i];
        const int j = (int) (e & PG_NBR_INDEX_MASK);
        const uint32_t code = e >> PG_NBR_INDEX_BITS;
        const double *base = a.p.pos;
        if(a.sync_ref && code != 0u) {
            int lag = gen_image_dims(code) - 1;
            lag = lag < a.list.steps_since_build ? lag : a.list.steps_since_build;
            base = lag <= 0 ? a.p.pos : (lag == 1 ? a.p.pos_prev1 : a.p.pos_prev2);
        }
        const double jx = gen_image(base[4 * (size_t) j], gen_shift(code, 0), a.box.len[0]);
        const double jy = gen_image(base[4 * (size_t) j + 1], gen_shift(code, 1), a.box.len[1]);
        const double jz = gen_image(base[4 * (size_t) j + 2], gen_shift(code, 2), a.box.len[2]);
        const double dx = xi_x - jx, dy = xi_y - jy, dz = xi_z - jz;
        const double rsq = ((dx * dx) + (dy * dy)) + (dz * dz);
        if(!(rsq < %(cutoff2)s)) { continue; }
%(body)s
    }
%(acc_store)s}
'''

PARTICLE = r'''
// particle kernel %(name)s
extern "C" __global__ void __launch_bounds__(256) k_%(name)s(GenArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= a.p.n) { return; }
%(filter)s%(body)s
}
'''

LAUNCH = r'''
extern "C" int run_%(name)s(const GenArgs *a, void *stream) {
    if(a->p.n <= 0) { return 0; }
    k_%(name)s<<<(a->p.n + 255) / 256, 256, 0, (cudaStream_t) stream>>>(*a);
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -2;
}
'''


class Module:
    def __init__(self, name, pair, cutoff, pre_step, skip_first, translator):
        self.name, self.pair, self.cutoff = name, pair, cutoff
        self.pre_step, self.skip_first = pre_step, skip_first
        self.applied = list(translator.applied)
        self.written = set(translator.written)
        self.read_j = set(translator.read_j)


def _kernel_source(name, tr, pair, cutoff, layout, setup=False):
    body = "\n".join("    " * (2 if pair else 0) + l for l in tr.lines)
    if not pair:
        # compute() kernels skip fixed particles (mapping/funcs.py:296-299); setup()
        # kernels run on every particle (mapping/funcs.py:356-359)
        filt = "" if setup else "    if(a.p.flags != nullptr && (a.p.flags[i] & 4)) { return; }\n"
        return PARTICLE % dict(name=name, body=body, filter=filt)
    decl, store = [], []
    for k, pname in enumerate(tr.applied):
        kind, base = layout.props[pname]
        if kind == VEC:
            decl.append(f"    double acc_{k}_x = 0.0, acc_{k}_y = 0.0, acc_{k}_z = 0.0;\n")
            for d, c in enumerate("xyz"):
                store.append(f"    if(a.half) {{ atomicAdd(&{base}[4 * (size_t) i + {d}], acc_{k}_{c}); }}\n"
                             f"    else {{ {base}[4 * (size_t) i + {d}] = {base}[4 * (size_t) i + {d}] + acc_{k}_{c}; }}\n")
        else:
            decl.append(f"    double acc_{k} = 0.0;\n")
            store.append(f"    if(a.half) {{ atomicAdd(&{base}[i], acc_{k}); }}\n"
                         f"    else {{ {base}[i] = {base}[i] + acc_{k}; }}\n")
    return PAIR % dict(name=name, cutoff=cutoff, cutoff2=c_literal(float(cutoff) * float(cutoff)),
                       body=body, acc_decl="".join(decl), acc_store="".join(store))


def lower_program(sim, entries):
    """entries: compute() records (func, cutoff, symbols, pre_step, skip_first) in
    program order.  Returns (modules, layout, CUDA source)."""
    if sim.position_prop is None:
        raise NotImplementedError("generated kernels need a position property")
    layout = Layout(sim)
    mods, parts = [], [PRELUDE % dict(max_props=MAX_PROPS, max_feat=MAX_FEATURES)]
    used = set()
    for e in entries:
        func = e["func"]
        nparams = len(inspect.signature(func).parameters)
        pair = nparams == 2
        if e.get("setup", False) and pair:
            raise NotImplementedError(f"{func.__name__}: setup functions take one parameter")
        if pair and e["cutoff"] is None:
            raise NotImplementedError(f"{func.__name__}: a pair kernel needs a cutoff radius")
        name = func.__name__
        while name in used:
            name += "_"
        used.add(name)
        tr = Translator(sim, layout, func, e["symbols"], pair)
        tr.indent = 1
        tr.body()
        parts.append(_kernel_source(name, tr, pair, e["cutoff"], layout, setup=e.get("setup", False)))
        parts.append(LAUNCH % dict(name=name))
        m = Module(name, pair, e["cutoff"], e.get("pre_step", False), e.get("skip_first", False), tr)
        m.setup = e.get("setup", False)
        mods.append(m)
    return mods, layout, "".join(parts)


def compile_source(source):
    """Compile the generated kernels into a shared library (cached by content)."""
    os.makedirs(GEN_DIR, exist_ok=True)
    key = hashlib.sha256(source.encode()).hexdigest()[:16]
    cu = os.path.join(GEN_DIR, f"gen_{key}.cu")
    so = os.path.join(GEN_DIR, f"libgen_{key}.so")
    if os.path.exists(so):
        return so
    with open(cu, "w") as f:
        f.write(source)
    from .build import nvcc, ARCH
    tmp = so + ".tmp"
    cmd = [nvcc(), "-shared", "-o", tmp, cu] + ARCH + ["-O3", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC",
                                                       "-I", os.path.join(ROOT, "include"), "-lcudart"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed on the generated kernels ({cu}):\n{res.stderr}")
    os.replace(tmp, so)
    return so
