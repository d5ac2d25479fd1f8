"""The update programs the engine generates for a system compile for sm_103a.

Runs on the CPU: code generation and NVRTC compilation need no GPU.  Every system
of the parser corpus is lowered through the library's parser (evolver level),
rebuilt at the solver level and its per-phase programs compiled, for 1D, 2D and
3D grids (line lengths 1, 16/32, 8)."""
import pytest

from tests.test_parser_parity import CORPUS


def solver_from_ir(ir, shape):
    import cupss_gb300 as c
    s = c.Solver(*shape, dt=0.01)
    names = [f["name"] for f in ir]
    for f in ir:
        s.add_field(f["dynamic"])
    for i, f in enumerate(ir):
        s.set_implicit(i, f["implicit"])
        for t in f["terms"]:
            s.add_term(i, [names.index(n) for n in t["product"]], t["pres"])
        if f["noisy"]:
            s.set_noise(i, f["noise"])
    return s


@pytest.mark.parametrize("shape", [(16, 1, 1), (32, 16, 1), (8, 4, 8)])
@pytest.mark.parametrize("case", range(len(CORPUS)))
def test_generated_programs_compile(built_lib, case, shape):
    import cupss_gb300 as c
    from cupss_gb300.api import jit_check
    from tests.test_parser_parity import build_lib
    ir = build_lib(*CORPUS[case])
    s = solver_from_ir(ir, shape)
    srcs = s.generated_sources()
    dyn = any(f["dynamic"] for f in ir)
    nd = any(not f["dynamic"] for f in ir)
    assert len(srcs) == int(dyn) + int(nd)
    for src in srcs:
        assert "cupssgb_turn" in src
        assert jit_check(src) > 0


@pytest.mark.parametrize("case", range(len(CORPUS)))
def test_batched_programs_compile(built_lib, case):
    """The batch variant (values from the member's row of the value table) compiles too."""
    from cupss_gb300.api import jit_check
    from tests.test_parser_parity import build_lib
    ir = build_lib(*CORPUS[case])
    s = solver_from_ir(ir, (32, 16, 1))
    s.set_members(8)
    for src in s.generated_sources():
        assert "P.mvals" in src and "P.pres[" not in src
        assert jit_check(src) > 0
    s.close()


def test_ensemble_declaration_errors(built_lib):
    """Errors the ensemble reports before touching a GPU."""
    import cupss_gb300 as c
    e = c.Ensemble()
    e.createField("h", True)
    e.addParameter("nu", 1.0)
    with pytest.raises(c.CupssError):
        e.createField("h", False)
    with pytest.raises(c.CupssError):
        e.addNoise("nope", "1")
    m = e.addMember(32, 32, 1, dt=0.01, seed=1)
    with pytest.raises(c.CupssError):
        e.setMemberParameter(m, "lam", 2.0)
    e.addEquation("dt h + nu*q^2*h = bogus*h")
    with pytest.raises(c.CupssError) as ex:
        e.prepare()
    assert ex.value.code == c.capi.ERR_PARSE
    e.close()


def test_server_declaration_errors(built_lib):
    """Errors the server reports on the caller's thread, before any GPU work."""
    import cupss_gb300 as c
    from cupss_gb300.workloads import SYSTEMS
    srv = c.Server(hbm_budget=1e9)
    sid = srv.addSystem(SYSTEMS["ew"])
    with pytest.raises(c.CupssError):
        srv.createField(sid, "h", True)
    with pytest.raises(c.CupssError):
        srv.setOutputField(sid, "nope")
    with pytest.raises(c.CupssError):
        srv.submit(sid, (32, 32, 1), 0.01, 10, params={"lam": 1.0})
    with pytest.raises(c.CupssError):
        srv.submit(sid + 5, (32, 32, 1), 0.01, 10)
    with pytest.raises(c.CupssError):
        srv.submit(sid, (32, 32, 1), 0.01, 0)
    srv.close()


@pytest.mark.parametrize("shape,split", [((64, 1024, 1), True), ((64, 512, 1), True), ((64, 256, 1), False),
                                         ((8, 8, 512), True), ((8, 8, 256), False)])
def test_turnaround_line_form(built_lib, shape, split):
    """Lines of 512 and 1024 points along the turnaround axis are generated in the split
    FFT form, shorter ones in the four-step form."""
    from cupss_gb300.api import jit_check
    from tests.test_parser_parity import build_lib
    ir = build_lib([("phi", 1)], {"a": -1.0, "b": 1.0, "k": 1.0, "T": 0.01},
                   ["dt phi + q^2*(a + k*q^2)*phi = -b*q^2*phi^3"], [("phi", "2*T*q^2")])
    s = solver_from_ir(ir, shape)
    (src,) = s.generated_sources()
    assert ("kSplit = %s;" % ("true" if split else "false")) in src
    assert jit_check(src) > 0


def test_member_memory_estimate(built_lib):
    """The device bytes a batch would allocate (the server's HBM-budget admission uses
    them): linear in the members, and at least the spectra a member needs: two states and
    one dealiased channel for phi, one product, 4 B per grid point each (packed half
    spectra)."""
    from tests.test_parser_parity import build_lib
    ir = build_lib([("phi", 1)], {"a": -1.0, "b": 1.0, "k": 1.0},
                   ["dt phi + q^2*(a + k*q^2)*phi = -b*q^2*phi^3"], [])
    for shape in ((64, 64, 1), (32, 16, 8)):
        s = solver_from_ir(ir, shape)
        e = [s.estimate_bytes(m) for m in (2, 3, 4, 8)]
        per = e[1] - e[0]
        assert e[2] - e[1] == per and e[3] - e[2] == 4 * per
        npts = shape[0] * shape[1] * shape[2]
        assert per >= 4 * 4 * npts
        assert s.estimate_bytes(1) > 0
        s.close()


KPZ_IR = ([("h", 1), ("iqxh", 0), ("iqyh", 0)], {"nu": 1.0, "lam": 1.0, "D": 1.0},
          ["dt h + nu*q^2*h = 0.5*lam*iqxh^2 + 0.5*lam*iqyh^2", "iqxh = iqx*h", "iqyh = iqy*h"],
          [("h", "2*D")])
CH_IR = ([("phi", 1)], {"a": -1.0, "b": 1.0, "k": 1.0, "T": 0.01},
         ["dt phi + q^2*(a + k*q^2)*phi = -b*q^2*phi^3"], [("phi", "2*T*q^2")])


def batched(ir, shape, members=4):
    s = solver_from_ir(ir, shape)
    s.set_members(members)
    return s


@pytest.mark.parametrize("system,shapes", [
    ("kpz", [(32, 32, 1), (64, 64, 1), (128, 128, 1), (256, 256, 1), (512, 512, 1), (1024, 1024, 1)]),
    ("kpz", [(64, 128, 1), (96, 96, 1), (384, 192, 1)]),
    ("ch", [(64, 64, 1), (1024, 512, 1), (96, 192, 1), (256, 1, 1), (2048, 1024, 1)]),
])
def test_fused_kernels_compile(built_lib, system, shapes):
    """The kernels that step several grid sizes in one launch per kernel (one body per
    grid, selected by block range) compile for sm_103a: phase 1 (products) holds a fused
    row pass and turnaround, phase 0 (KPZ's iqxh, iqyh) a fused turnaround."""
    from cupss_gb300.api import jit_check, multi_generated_sources
    from tests.test_parser_parity import build_lib
    ir = build_lib(*(KPZ_IR if system == "kpz" else CH_IR))
    solvers = [batched(ir, sh) for sh in shapes]
    src0, src1 = multi_generated_sources(solvers)
    assert bool(src0) == (system == "kpz")
    assert "cupssgb_turn_multi" in src1 and "cupssgb_row_multi" in src1
    for c in range(len(shapes)):
        assert "MP.span[%d]" % c in src1
    for src in (src0, src1):
        if src:
            assert jit_check(src) > 0
    for s in solvers:
        s.close()


def test_fused_refusals(built_lib):
    """3D grids, different systems, plain (unbatched) solvers and rows whose pass needs
    another block shape are not fused (the ensemble then steps each grid on its own)."""
    import cupss_gb300 as c
    from cupss_gb300.api import multi_generated_sources
    from tests.test_parser_parity import build_lib
    kpz, ch = build_lib(*KPZ_IR), build_lib(*CH_IR)
    cases = [([batched(ch, (32, 32, 1)), batched(ch, (16, 16, 16))], "1D and 2D"),
             ([batched(ch, (32, 32, 1)), batched(kpz, (64, 64, 1))], "structure"),
             ([batched(ch, (32, 32, 1)), solver_from_ir(ch, (64, 64, 1))], "batched"),
             # rows of sx = 48 take a row-pass block other than the fused one's 128 threads
             ([batched(ch, (48, 192, 1)), batched(ch, (64, 64, 1))], "row pass block")]
    for solvers, why in cases:
        with pytest.raises(c.CupssError) as ex:
            multi_generated_sources(solvers)
        assert why in str(ex.value), str(ex.value)
        for s in solvers:
            s.close()


@pytest.mark.parametrize("merge", [True, False])
def test_product_terms_with_equal_prefactors_share_a_channel(built_lib, monkeypatch, merge):
    """KPZ's 0.5*lam*iqxh^2 + 0.5*lam*iqyh^2: with merging the row pass sums the two
    squares in real space and the update reads one product channel (the second term is
    skipped); CUPSSGB_MERGE=0 keeps one channel per product."""
    from cupss_gb300.api import jit_check
    from tests.test_parser_parity import build_lib
    if not merge:
        monkeypatch.setenv("CUPSSGB_MERGE", "0")
    s = solver_from_ir(build_lib(*KPZ_IR), (64, 64, 1))
    src0, src1 = s.generated_sources()
    assert "fx.prod(0)" in src1
    assert ("fx.prod(1)" in src1) != merge
    assert "kNProd = %d;" % (1 if merge else 2) in src1
    assert jit_check(src1) > 0
    s.close()


def test_merge_needs_equal_prefactors_and_exclusive_products(built_lib):
    """Model H: phi's -vx*iqxphi - vy*iqyphi (equal prefactors) share a channel; phi^3
    (another prefactor) and the velocity equations' products (each used by two terms with
    different prefactors) keep their own."""
    from tests.test_parser_parity import build_lib
    fields = [("phi", 1), ("iqxphi", 0), ("iqyphi", 0), ("lapphi", 0), ("vx", 0), ("vy", 0)]
    eqs = ["dt phi + q^2*(a + k*q^2)*phi = -b*q^2*phi^3 - vx*iqxphi - vy*iqyphi",
           "iqxphi = iqx*phi", "iqyphi = iqy*phi", "lapphi = -q^2*phi",
           "vx*eta*q^2 = -k*iqxphi*lapphi - k*iqx^2*1/q^2*iqxphi*lapphi - k*iqx*iqy*1/q^2*iqyphi*lapphi",
           "vy*eta*q^2 = -k*iqyphi*lapphi - k*iqy^2*1/q^2*iqyphi*lapphi - k*iqx*iqy*1/q^2*iqxphi*lapphi"]
    ir = build_lib(fields, {"a": -1.0, "b": 1.0, "k": 4.0, "eta": 1.0, "T": 0.001}, eqs, [("phi", "2*T")])
    s = solver_from_ir(ir, (64, 64, 1))
    src0, src1 = s.generated_sources()
    assert "kNProd = 2;" in src1    # phi^3, and vx*iqxphi + vy*iqyphi
    assert "kNProd = 2;" in src0    # iqxphi*lapphi, iqyphi*lapphi: each used with several prefactors
    s.close()


@pytest.mark.parametrize("b,merged", [(1.0, True), (2.0, False)])
def test_merge_only_with_identical_prefactors(built_lib, b, merged):
    """dt phi = a*phi^2 + b*psi^2: one channel when a == b, two otherwise; in a batch, one
    member with a different b keeps the products apart for all."""
    from tests.test_parser_parity import build_lib
    ir = build_lib([("phi", 1), ("psi", 1)], {"a": 1.0, "b": b},
                   ["dt phi + q^2*phi = a*phi^2 + b*psi^2", "dt psi + q^2*psi = 0"], [])
    s = solver_from_ir(ir, (32, 32, 1))
    src = s.generated_sources()[0]
    assert ("kNProd = 1;" in src) == merged
    s.close()
    if merged:
        from cupss_gb300.capi import Pres
        s = solver_from_ir(ir, (32, 32, 1))
        s.set_members(3)
        fi = [f["name"] for f in ir].index("phi")
        t = [i for i, term in enumerate(ir[fi]["terms"]) if term["product"] == ["psi", "psi"]][0]
        pres = ir[fi]["terms"][t]["pres"]
        s.set_member_term_pres(2, fi, t, [Pres(p[0] * 3.0, *p[1:]) for p in pres])
        assert "kNProd = 2;" in s.generated_sources()[0]
        s.close()


def test_merge_groups_only_exclusive_products(built_lib):
    """phi: a*phi^2 + a*psi^2 + c*phi*psi; psi: a*psi^2.  psi^2 is used by both fields, so
    only phi^2 could merge -- and alone it stays its own channel: three channels.  With
    psi's term removed, phi^2 and psi^2 (equal prefactors) share one: two channels."""
    from tests.test_parser_parity import build_lib
    params = {"a": 1.0, "c": 2.0}
    shared = build_lib([("phi", 1), ("psi", 1)], params,
                       ["dt phi + q^2*phi = a*phi^2 + a*psi^2 + c*phi*psi", "dt psi + q^2*psi = a*psi^2"], [])
    s = solver_from_ir(shared, (32, 32, 1))
    assert "kNProd = 3;" in s.generated_sources()[0]
    s.close()
    alone = build_lib([("phi", 1), ("psi", 1)], params,
                      ["dt phi + q^2*phi = a*phi^2 + a*psi^2 + c*phi*psi", "dt psi + q^2*psi = 0"], [])
    s = solver_from_ir(alone, (32, 32, 1))
    src = s.generated_sources()[0]
    assert "kNProd = 2;" in src
    from cupss_gb300.api import jit_check
    assert jit_check(src) > 0
    s.close()


def test_fused_block_ranges_cover_every_tile(built_lib):
    """The fused turnaround's blockIdx.x ranges: contiguous, one per grid class, each as
    long as ceil((sx/2) / W_c) for the class's tile width W_c, and W_c * M_c the same
    thread count for every class (M_c threads per line); the row pass's ranges hold
    ceil(sy / RW_c) blocks of 128 threads (M_c * RW_c = 128)."""
    import re
    from cupss_gb300.api import multi_generated_sources
    from tests.test_parser_parity import build_lib
    shapes = [(512, 512, 1), (256, 256, 1), (96, 96, 1), (256, 1, 1), (64, 128, 1)]
    solvers = [batched(build_lib(*KPZ_IR), sh) for sh in shapes]
    _, src = multi_generated_sources(solvers)
    turn = src[src.index("cupssgb_turn_multi"):src.index("cupssgb_row_multi")]
    row = src[src.index("cupssgb_row_multi"):]
    threads = int(re.search(r"__launch_bounds__\((\d+), \d+\) cupssgb_turn_multi", src).group(1))
    ends = [int(x) for x in re.findall(r"if \(bx < (\d+)\)", turn)]
    calls = re.findall(r"turn_body_at<(\d+), 1, [^>]*>\(MP\.p\[(\d)\], bx - (\d+), 0, tid % (\d+), tid / (\d+), 0\)",
                       turn)
    assert len(ends) == len(calls) == len(shapes)
    start = 0
    for c, ((L, idx, b0, W, W2), end, (sx, sy, sz)) in enumerate(zip(calls, ends, shapes)):
        assert int(idx) == c and int(b0) == start and W == W2 and int(L) == sy
        W = int(W)
        assert threads % W == 0
        assert end - start == -(-(sx // 2) // W), (c, end - start, sx, W)
        start = end
    rends = [int(x) for x in re.findall(r"if \(bx < (\d+)\)", row)]
    rcalls = re.findall(r"(row_one_body|row_pass_body)<(\d+), (true|false)>\(MP\.x\[(\d)\], bx - (\d+), tid % (\d+), "
                        r"tid / (\d+)\)", row)
    assert len(rends) == len(rcalls) == len(shapes)
    start = 0
    for c, ((_, LX, _, idx, b0, M, M2), end, (sx, sy, sz)) in enumerate(zip(rcalls, rends, shapes)):
        assert int(idx) == c and int(b0) == start and M == M2 and int(LX) == sx // 2
        rw = 128 // int(M)
        assert end - start == -(-(sy * sz) // rw), (c, end - start, sy, rw)
        start = end
    for s in solvers:
        s.close()
