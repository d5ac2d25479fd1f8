"""Oracle restatement of cuPSS's equation parser (TEST INFRASTRUCTURE ONLY).

This module is part of the CPU oracle.  Only ``tests/``, ``__graft_entry__.smoke``
and the CPU-baseline leg of ``bench.py`` may import it; the product (the C++ host
library and its CUDA engine) never does.

It restates, in plain Python, the string -> IR lowering of the reference parser
(src/parser.cpp), including its quirks, so that the C++ parser shipped by this
project can be checked against it equation by equation:

* ``remove_spaces``           src/parser.cpp:433-447
* ``split_equation_sides``    src/parser.cpp:406-431
* ``split_terms``             src/parser.cpp:449-474   (top-level +/- split)
* ``expand_once/expand_all``  src/parser.cpp:477-545   (parenthesis distribution)
* ``get_factors``             src/parser.cpp:355-377
* ``is_number``               src/parser.cpp:125-155
* ``is_numerical_factor``     src/parser.cpp:157-196
* ``is_field``                src/parser.cpp:199-227
* ``is_q2n_factor``           src/parser.cpp:229-245   (q^3 -> 3/2 = 1, C division)
* ``is_iq_factor``            src/parser.cpp:247-267
* ``get_prefactor``           src/parser.cpp:547-589
* ``get_field_vector``        src/parser.cpp:591-626
* ``add_equation``            src/parser.cpp:628-767   (implicit/explicit split,
                                                        grouping by sorted field multiset,
                                                        trivial-implicit drop at :728)
* ``add_noise``               src/parser.cpp:379-404
* ``isParameterInString``     src/parser.cpp:811-835

Fatal parse errors (the reference prints and ``exit(1)``s) raise ``ParseError``.
"""
from __future__ import annotations

from dataclasses import dataclass, field as dc_field
from typing import Dict, List


class ParseError(Exception):
    pass


@dataclass
class Pres:
    """One q-monomial prefactor; same fields as ``struct pres`` (inc/cupss/defines.h:31-39)."""
    pre: float = 0.0
    q2n: int = 0
    iqx: int = 0
    iqy: int = 0
    iqz: int = 0
    invq: int = 0

    def key(self):
        return (self.pre, self.q2n, self.iqx, self.iqy, self.iqz, self.invq)


@dataclass
class Term:
    """One explicit RHS group: product of fields (sorted multiset) times a sum of pres."""
    product: List[str]
    pres: List[Pres]
    strings: List[str] = dc_field(default_factory=list)


@dataclass
class FieldIR:
    name: str
    dynamic: bool
    implicit: List[Pres] = dc_field(default_factory=list)
    implicit_strings: List[str] = dc_field(default_factory=list)
    terms: List[Term] = dc_field(default_factory=list)
    noisy: bool = False
    noise: Pres = dc_field(default_factory=Pres)


def _f32(x: float) -> float:
    import numpy as np
    return float(np.float32(x))


def _c_atoi(s: str) -> int:
    """C ``atoi``: optional sign then leading digits, 0 if none."""
    i, n = 0, len(s)
    while i < n and s[i] in " \t\n":
        i += 1
    sign = 1
    if i < n and s[i] in "+-":
        sign = -1 if s[i] == "-" else 1
        i += 1
    v = 0
    while i < n and s[i].isdigit():
        v = v * 10 + int(s[i])
        i += 1
    return sign * v


def _c_div(a: int, b: int) -> int:
    q = abs(a) // abs(b)
    return q if (a >= 0) == (b > 0) else -q


class System:
    """Holds fields and parameters like the reference ``evolver`` + ``parser`` pair."""

    def __init__(self):
        self.fields: Dict[str, FieldIR] = {}
        self.order: List[str] = []
        self.parameters: Dict[str, float] = {}

    # ---- registry -------------------------------------------------------------
    def create_field(self, name: str, dynamic: bool) -> int:
        if name in self.fields:
            return 1
        self.fields[name] = FieldIR(name, bool(dynamic))
        self.order.append(name)
        return 0

    def add_parameter(self, name: str, value: float) -> int:
        if name in self.parameters:
            return -1
        self.parameters[name] = _f32(value)
        return 0

    # ---- lexical helpers ----------------------------------------------------------
    @staticmethod
    def remove_spaces(s: str) -> str:
        return s.replace(" ", "")

    @staticmethod
    def split_terms(s: str) -> List[str]:
        out, cur, level = [], 0, 0
        for p, ch in enumerate(s):
            if ch == "(":
                level += 1
            if ch == ")":
                level -= 1
            if p > 0 and level == 0 and ch in "+-":
                out.append(s[cur:p])
                cur = p
        out.append(s[cur:])
        return out

    @classmethod
    def expand_once(cls, s: str):
        level, found, cur = 0, False, 0
        for p, ch in enumerate(s):
            if ch == "(":
                if p > 0 and s[p - 1] == "/":
                    raise ParseError("No dividing over parenthesis allowed!")
                found = True
                level += 1
                if level == 1:
                    cur = p
            if ch == ")":
                level -= 1
            if level == 0 and found:
                inner = cls.split_terms(s[cur + 1:p])
                pre, post = s[:cur], s[p + 1:]
                res = []
                for t in inner:
                    this_pre = pre
                    if t[:1] == "+":
                        t = t[1:]
                    if t[:1] == "-":
                        if this_pre[:1] == "-":
                            this_pre = "+" + this_pre[1:]
                        elif this_pre[:1] == "+":
                            this_pre = "-" + pre[1:]
                        else:
                            this_pre = "-" + this_pre
                        t = t[1:]
                    res.append(this_pre + t + post)
                return res
        return None

    @classmethod
    def expand_all(cls, terms: List[str]) -> List[str]:
        terms = list(terms)
        k = 0
        while k < len(terms):
            sub = cls.expand_once(terms[k])
            if sub is not None:
                del terms[k]
                terms.extend(sub)
                continue
            k += 1
        return terms

    @staticmethod
    def get_factors(s: str) -> List[str]:
        out, start, opened = [], 0, 0
        for p, ch in enumerate(s):
            if ch == "(":
                opened = 1
            if ch == ")":
                opened = 0
            if ch == "*" and opened == 0:
                out.append(s[start:p])
                start = p + 1
            if p == len(s) - 1:
                out.append(s[start:])
        return out

    # ---- factor classification ------------------------------------------------------
    @staticmethod
    def is_number(term: str) -> bool:
        t = term[2:] if term[:2] == "1/" else term
        periods = [i for i, c in enumerate(t) if c == "."]
        if len(periods) > 1:
            raise ParseError("prefactor not a parameter and not a number: " + term)
        if periods:
            i = periods[-1]
            t = t[:i] + t[i + 1:]
        return all(c.isdigit() for c in t)

    def is_field(self, factor: str) -> int:
        power, ppos = 1, 0
        for i, c in enumerate(factor):
            if c == "^":
                power = _c_atoi(factor[i + 1:])
                ppos = i
        if power != 1:
            return power if factor[:ppos] in self.fields else 0
        return power if factor in self.fields else 0

    def is_q2n_factor(self, factor: str) -> int:
        if len(factor) < 3:
            return 0
        if factor[0] == "q" and factor[1] == "^":
            num = factor[2:]
            if not self.is_number(num):
                raise ParseError(num + " power of q not a number, missing *?")
            return _c_atoi(num)
        return 0

    def is_iq_factor(self, factor: str, iq: str) -> int:
        if len(factor) < 3:
            return 0
        if factor[:3] == iq and len(factor) == 3:
            return 1
        if factor[:3] == iq:
            num = factor[4:]
            if not self.is_number(num):
                raise ParseError(num + " power of " + iq + " not a number, missing *?")
            return _c_atoi(num)
        return 0

    def is_numerical_factor(self, factor: str) -> float:
        if self.is_q2n_factor(factor):
            return 1.0
        for iq in ("iqx", "iqy", "iqz", "1/q"):
            if self.is_iq_factor(factor, iq):
                return 1.0
        if self.is_field(factor):
            return 1.0
        divides = factor[:2] == "1/"
        f = factor[2:] if divides else factor
        if f in self.parameters:
            v = self.parameters[f]
            return _f32(1.0 / v) if divides else v
        if self.is_number(f):
            try:
                v = _f32(float(f))
            except ValueError:
                raise ParseError("parameter not found and not a number: " + factor)
            return _f32(1.0 / v) if divides else v
        raise ParseError("parameter not found and not a number: " + factor)

    # ---- term-level ---------------------------------------------------------------------
    @staticmethod
    def _insert_div_marks(t: str) -> str:
        out = []
        for c in t:
            if c == "/":
                out.append("*1")
            out.append(c)
        return "".join(out)

    def get_prefactor(self, term: str) -> Pres:
        p = Pres(1.0)
        if term[:1] == "+":
            term = term[1:]
        if term[:1] == "-":
            p.pre = -1.0
            term = term[1:]
        term = self._insert_div_marks(term)
        for f in self.get_factors(term):
            if self.is_field(f) > 0:
                continue
            p.pre = _f32(p.pre * self.is_numerical_factor(f))
            p.q2n += _c_div(self.is_q2n_factor(f), 2)
            p.iqx += self.is_iq_factor(f, "iqx")
            p.iqy += self.is_iq_factor(f, "iqy")
            p.iqz += self.is_iq_factor(f, "iqz")
            p.invq += self.is_iq_factor(f, "1/q")
        return p

    def extract_field_name(self, t: str) -> str:
        if self.is_field(t) == 1:
            return t
        chev = 0
        for i, c in enumerate(t):
            if c == "^":
                chev = i
        return t[:chev]

    def get_field_vector(self, term: str) -> List[str]:
        if term[:1] == "+":
            term = term[1:]
        if term[:1] == "-":
            term = term[1:]
        term = self._insert_div_marks(term)
        out = []
        for f in self.get_factors(term):
            n = self.is_field(f)
            if n > 0:
                out.extend([self.extract_field_name(f)] * n)
        return out

    def number_of_fields(self, term: str) -> int:
        if term[:1] in ("+", "-"):
            term = term[1:]
        return sum(self.is_field(f) for f in self.get_factors(term))

    def get_field_name(self, term: str) -> str:
        if term[:1] in ("+", "-"):
            term = term[1:]
        name = ""
        for f in self.get_factors(term):
            if self.is_field(f) > 0:
                name = f
        return name

    def is_parameter_in_string(self, s: str, param: str) -> int:
        loc = s[1:] if s[:1] in ("+", "-") else s
        loc = loc.replace("/", "*")
        return sum(1 for f in self.get_factors(loc) if f == param)

    # ---- equations ------------------------------------------------------------------------
    def add_equation(self, equation: str) -> int:
        eq = self.remove_spaces(equation)
        if eq.count("=") != 1:
            raise ParseError("More than one equal sign")
        pos = eq.index("=")
        lhs, rhs = eq[:pos], eq[pos + 1:]
        lhs_terms = self.expand_all(self.split_terms(lhs))
        rhs_terms = self.expand_all(self.split_terms(rhs))
        dynamic = False
        if lhs_terms[0][:2] == "dt":
            dynamic = True
            name = lhs_terms[0][2:]
            if not self.is_field(name):
                raise ParseError("Field not found: " + name)
            if self.is_field(name) > 1:
                raise ParseError("Nonlinearity in lhs: " + name)
            lhs_terms = lhs_terms[1:]
        else:
            if self.number_of_fields(lhs_terms[0]) != 1:
                raise ParseError("Nonlinear term in left hand side")
            name = self.get_field_name(lhs_terms[0])
        implicits = []
        for t in lhs_terms:
            fv = self.get_field_vector(t)
            if len(fv) != 1:
                raise ParseError("Nonlinear term in lhs")
            if fv[0] != name:
                raise ParseError(name + " and " + fv[0] + " incompatible in lhs")
            p = self.get_prefactor(t)
            if dynamic:
                p.pre = _f32(-p.pre)
            implicits.append(p)
        groups: List[List[str]] = []
        group_pres: List[List[Pres]] = []
        group_str: List[List[str]] = []
        for t in rhs_terms:
            fv = sorted(self.get_field_vector(t))
            p = self.get_prefactor(t)
            hit = False
            for k, g in enumerate(groups):
                if g == fv:
                    hit = True
                    group_pres[k].append(p)
                    group_str[k].append(t)
            if not hit:
                groups.append(fv)
                group_pres.append([p])
                group_str.append([t])
        fld = self.fields[name]
        trivial = (len(implicits) == 1 and implicits[0].key() == (1.0, 0, 0, 0, 0, 0))
        if not trivial:
            for p, s in zip(implicits, lhs_terms):
                fld.implicit.append(p)
                fld.implicit_strings.append(s)
        for g, ps, ss in zip(groups, group_pres, group_str):
            fld.terms.append(Term(list(g), list(ps), list(ss)))
        return 0

    def add_noise(self, name: str, equation: str) -> int:
        if name not in self.fields:
            return -1
        eq = self.remove_spaces(equation)
        p = Pres(1.0)
        for f in self.get_factors(eq):
            p.pre = _f32(p.pre * self.is_numerical_factor(f))
            p.q2n += _c_div(self.is_q2n_factor(f), 2)
            p.invq += self.is_iq_factor(f, "1/q")
        fld = self.fields[name]
        fld.noisy = True
        fld.noise = p
        return 0

    def update_parameter(self, name: str, value: float) -> None:
        """Re-derives the pres of every string that mentions ``name``
        (src/evolver.cpp:386-394, src/field.cpp:422-441, src/parser.cpp:838-846)."""
        if name not in self.parameters:
            raise ParseError("changeParameter " + name + " not found")
        self.parameters[name] = _f32(value)
        for fld in self.fields.values():
            if any(self.is_parameter_in_string(s, name) for s in fld.implicit_strings):
                for i, s in enumerate(fld.implicit_strings):
                    p = self.get_prefactor(s)
                    if fld.dynamic:
                        p.pre = _f32(-p.pre)
                    fld.implicit[i] = p
            for t in fld.terms:
                if any(self.is_parameter_in_string(s, name) for s in t.strings):
                    t.pres = [self.get_prefactor(s) for s in t.strings]

    # ---- export ---------------------------------------------------------------------------------
    def ir(self):
        """Plain-data IR: list of dicts in field creation order (product names resolved)."""
        out = []
        for n in self.order:
            f = self.fields[n]
            out.append({
                "name": f.name, "dynamic": f.dynamic,
                "implicit": [list(p.key()) for p in f.implicit],
                "terms": [{"product": list(t.product), "pres": [list(p.key()) for p in t.pres]}
                          for t in f.terms],
                "noisy": f.noisy, "noise": list(f.noise.key()),
            })
        return out
