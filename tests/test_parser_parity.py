"""The library's C++ parser lowers equations to the same IR as the oracle's
restatement of the reference parser (src/parser.cpp:628-767).

Runs on the CPU: parsing needs no GPU.  The corpus holds every equation of the
reference examples and tests plus corner cases of the grammar.
"""
import numpy as np
import pytest

from oracle.ref_parser import System, ParseError

CORPUS = [
    # (fields [(name, dynamic)], params {name: value}, equations, noises [(field, amp)])
    ([("phi", 1)], {"a": -1, "b": 1, "k": 1}, ["dt phi + q^2*(a + k*q^2)*phi = -b*q^2*phi^3"], []),
    ([("phi", 1)], {"a": -1, "b": 1, "k": 4}, ["dt phi + ( a *q^2 + k*q^4)*phi= - b* q^2* phi^3 "], []),
    ([("phi", 1)], {"a": -1.0, "b": 1.0, "k": 4.0, "D": 1.0},
     ["dt phi + q^2*(a + k*q^2)*phi= - b*q^2*phi^3"], [("phi", "2*D*q^2")]),
    ([("phi", 1)], {"D": 1.0}, ["dt phi + D * q^2 * phi = 0"], [("phi", "2*D")]),
    ([("h", 1), ("iqh", 0)], {"D": 0.5, "l": 0.5},
     ["dt h + 0.5 * q^2 * h = l * iqh^2", "iqh = iqx*h"], [("h", "2*D")]),
    ([("h", 1), ("iqxh", 0), ("iqyh", 0)], {"nu": 1.3, "lambda": 2.0, "D": 1.0},
     ["dt h + nu*q^2*h = 0.5*lambda*iqxh^2 + 0.5*lambda*iqyh^2", "iqxh = iqx*h", "iqyh = iqy*h"],
     [("h", "2*D")]),
    ([("phi", 1), ("iqxphi", 0), ("iqyphi", 0), ("sigxx", 0), ("sigxy", 0), ("vx", 0), ("vy", 0), ("w", 0)],
     {"a": -1.0, "b": 1.0, "k": 4.0, "eta": 1.0, "friction": 0.0, "ka": -4.0, "D": 0.01},
     ["dt phi + ( a *q^2 + k*q^4)*phi= - b* q^2* phi^3 -vx*iqxphi - vy*iqyphi",
      "iqxphi = iqx*phi", "iqyphi = iqy*phi",
      "sigxx = - 0.5*ka *iqxphi * iqxphi + 0.5*ka*iqyphi*iqyphi",
      "sigxy = - ka *iqxphi * iqyphi",
      "vx * (friction + eta*q^2) = (iqx + iqx^3*1/q^2 - iqx*iqy^2*1/q^2) * sigxx + (iqy + iqx^2* iqy*1/q^2 + iqx^2*iqy*1/q^2) * sigxy",
      "vy * (friction + eta*q^2) = (iqx + iqx*iqy^2*1/q^2 + iqx*iqy^2*1/q^2) * sigxy + (-iqy - iqy^3*1/q^2 + iqx^2*iqy*1/q^2) * sigxx",
      "w = 0.5*iqx * vy - 0.5*iqy*vx "], []),
    ([("phi", 1), ("iqxphi", 0), ("iqyphi", 0), ("sigxx", 0), ("sigxy", 0), ("vx", 0), ("vy", 0), ("w", 0), ("P", 0)],
     {"a": -1.0, "b": 1.0, "k": 4.0, "eta": 1.0, "friction": 0.0, "ka": 4.0},
     ["dt phi + ( a *q^2 + k*q^4)*phi= - b* q^2* phi^3 -vx*iqxphi - vy*iqyphi",
      "iqxphi = iqx*phi", "iqyphi = iqy*phi",
      "sigxx = - 0.5*ka *iqxphi * iqxphi + 0.5*ka*iqyphi*iqyphi", "sigxy = - ka *iqxphi * iqyphi",
      "-q^2*P = (iqx*iqx-iqy*iqy)*sigxx + 2.0 * iqx*iqy*sigxy",
      "vx * (friction + eta*q^2) = -iqx*P + iqx*sigxx + iqy*sigxy",
      "vy * (friction + eta*q^2) = -iqy*P + iqx*sigxy - iqy*sigxx",
      "w = 0.5*iqx * vy - 0.5*iqy*vx "], []),
    ([("phi", 1), ("iqxphi", 0), ("iqyphi", 0), ("lapphi", 0), ("vx", 0), ("vy", 0)],
     {"a": -1.0, "b": 1.0, "k": 4.0, "eta": 1.0, "T": 0.001},
     ["dt phi + q^2*(a + k*q^2)*phi = -b*q^2*phi^3 - vx*iqxphi - vy*iqyphi",
      "iqxphi = iqx*phi", "iqyphi = iqy*phi", "lapphi = -q^2*phi",
      "vx*eta*q^2 = -k*iqxphi*lapphi - k*iqx^2*1/q^2*iqxphi*lapphi - k*iqx*iqy*1/q^2*iqyphi*lapphi",
      "vy*eta*q^2 = -k*iqyphi*lapphi - k*iqy^2*1/q^2*iqyphi*lapphi - k*iqx*iqy*1/q^2*iqxphi*lapphi"],
     [("phi", "2*T")]),
    ([("v", 1), ("iqxv", 0), ("x", 0)], {}, ["dt v +0.5*q^2*v = iqx*x*iqxv + x*iqy^2*v", "iqxv = iqx*v"], []),
    ([("phi_gpu_3d", 1), ("lapphi_gpu_3d", 0), ("iqxphi_gpu_3d", 0), ("iqyphi_gpu_3d", 0),
      ("iqzphi_gpu_3d", 0), ("invqphi_gpu_3d", 0)], {},
     ["dt phi_gpu_3d +q^2*phi_gpu_3d = iqxphi_gpu_3d^2", "lapphi_gpu_3d = -q^2*phi_gpu_3d",
      "iqxphi_gpu_3d =  iqx*phi_gpu_3d", "iqyphi_gpu_3d =  iqy*phi_gpu_3d",
      "iqzphi_gpu_3d =  iqz*phi_gpu_3d", "invqphi_gpu_3d =  1/q*phi_gpu_3d"], []),
    # corner cases: divisions, nested parentheses, negative groups, q^3 (3/2 = 1), constants,
    # trivial implicit dropped even for a dynamic field written "dt f - f"
    ([("u", 1), ("v", 0)], {"a": 2.0, "b": 4.0},
     ["dt u - u = a/b*u - (a*(q^2 - 1/q))*v + 3*q^3*u^2*v - (-(b*iqz))*v + 2.5",
      "v*(1 + a*q^2) = u/a + 1/q^2*u"], [("u", "a*q^2*1/q")]),
    ([("u", 1)], {}, ["dt u = "], []),
]


def build_oracle(fields, params, eqs, noises):
    s = System()
    for n, d in fields:
        s.create_field(n, bool(d))
    for k, v in params.items():
        s.add_parameter(k, v)
    for e in eqs:
        s.add_equation(e)
    for f, a in noises:
        s.add_noise(f, a)
    return s.ir()


def build_lib(fields, params, eqs, noises):
    import cupss_gb300 as c
    e = c.Evolver(True, 8, 8, 1)
    for n, d in fields:
        e.createField(n, bool(d))
    for k, v in params.items():
        e.addParameter(k, v)
    for q in eqs:
        e.addEquation(q)
    for f, a in noises:
        e.addNoise(f, a)
    return e.describe()


def norm(ir):
    out = []
    for f in ir:
        out.append((f["name"], bool(f["dynamic"]),
                    [tuple(np.float32(p[0]).item() if i == 0 else int(p[i]) for i in range(6)) for p in f["implicit"]],
                    [(tuple(t["product"]), [tuple(np.float32(p[0]).item() if i == 0 else int(p[i]) for i in range(6))
                                            for p in t["pres"]]) for t in f["terms"]],
                    bool(f["noisy"]),
                    tuple(np.float32(f["noise"][0]).item() if i == 0 else int(f["noise"][i]) for i in range(6))
                    if f["noisy"] else None))
    return out


@pytest.mark.parametrize("case", range(len(CORPUS)))
def test_cpp_parser_matches_oracle(built_lib, case):
    fields, params, eqs, noises = CORPUS[case]
    assert norm(build_lib(fields, params, eqs, noises)) == norm(build_oracle(fields, params, eqs, noises))


@pytest.mark.parametrize("bad", ["dt phi = = 1", "dt phi + phi^2 = 0", "dt phi = unknown*phi",
                                 "dt phi = 1/(q^2)*phi", "dt phi = q^x*phi", "dt psi = phi"])
def test_parse_errors_reported(built_lib, bad):
    import cupss_gb300 as c
    s = System()
    s.create_field("phi", True)
    with pytest.raises(ParseError):
        s.add_equation(bad)
    e = c.Evolver(True, 8, 8, 1)
    e.createField("phi", True)
    with pytest.raises(c.CupssError) as ei:
        e.addEquation(bad)
    assert ei.value.code == -5


def test_update_parameter_rederives_pres(built_lib):
    import cupss_gb300 as c
    eqs = ["dt phi + q^2*(a + k*q^2)*phi = -b*q^2*phi^3"]
    e = c.Evolver(True, 8, 8, 1)
    e.createField("phi", True)
    for k, v in {"a": -1, "b": 1, "k": 1}.items():
        e.addParameter(k, v)
    e.addEquation(eqs[0])
    s = System()
    s.create_field("phi", True)
    for k, v in {"a": -1, "b": 1, "k": 1}.items():
        s.add_parameter(k, v)
    s.add_equation(eqs[0])
    e.updateParameter("b", 3.0)
    s.update_parameter("b", 3.0)
    assert norm(e.describe()) == norm(s.ir())
    assert abs(e.getParameter("b") - 3.0) < 1e-7
