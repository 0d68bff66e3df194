"""The C-ABI library builds, loads and exports every entry point of include/sfdx.h (no GPU needed)."""
import ctypes
import os
import re

import numpy as np

import sfd_excmg_gb300 as S
from oracle import oracle as O
from sfd_excmg_gb300 import capi
from sfd_excmg_gb300 import synthetic as syn

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "sfdx.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(sfdx_\w+)\s*\(", src)))


def test_every_declared_symbol_is_exported(lib):
    names = _declared()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
    for n in names:
        assert n in capi._PROTO, f"{n} has no ctypes prototype"


def test_binding_declares_nothing_beyond_the_header():
    """The ctypes prototypes are exactly the entry points the header declares."""
    extra = sorted(set(capi._PROTO) - set(_declared()))
    assert not extra, extra


def test_default_options_match_reference_constants():
    o = S.Opts.defaults()
    assert (o.level, o.solver, o.excmg, chr(o.precond)) == (3, 1, 0, "S")
    assert (o.div_cor, o.corr_intv, o.corr_tol, o.ssor_omega) == (1, 200, 1e-3, 1.0)
    assert (o.sigma_air, o.maxit_plain, o.maxit_level) == (1e-9, 5000, 1000)
    assert o.quirks == capi.QUIRKS_REFERENCE
    assert ctypes.sizeof(S.Opts) == ctypes.sizeof(capi.Opts)


def test_strerror_covers_codes(lib):
    for code in range(0, 11):
        assert len(lib.sfdx_strerror(code)) > 0


def test_host_mt1d_matches_oracle():
    m = syn.small_aniso()
    conv = O.column_conv(m.sigma, m.nx, m.ny, m.nz)
    conv[:, 3] = 0.2 * conv[:, 0]
    conv[:, 4] = 0.1 * conv[:, 0]
    conv[:, 5] = -0.15 * conv[:, 0]
    for f in (1e-3, 1.0, 1e3):
        e1, h1, i1 = O.mt1d_anl(f, conv, m.c)
        e2, h2, i2 = S.mt1d(f, conv, m.c)
        np.testing.assert_allclose(e2, e1, rtol=1e-13, atol=1e-15)
        np.testing.assert_allclose(h2, h1, rtol=1e-13, atol=1e-30)
        np.testing.assert_allclose(i2, i1, rtol=1e-13)


def test_host_impedance_matches_post_process():
    m = syn.small_aniso(freqs=(0.1, 10.0))
    rng = np.random.default_rng(0)
    ex = rng.standard_normal((2, 2, m.nl)) + 1j * rng.standard_normal((2, 2, m.nl))
    om = O.OracleModel(m.nx, m.ny, m.nz, m.nair, m.a, m.b, m.c, m.sigma, m.freq, m.recv)
    for out_type, rd, q in ((1, 2, 7), (2, 1, 3), (0, 2, 4)):
        ref = O.impedances(om, ex, out_type=out_type, rd=rd)
        got, tip = S.impedance(m, ex, out_type=out_type, quirks=q, tipper=True)
        np.testing.assert_allclose(got, ref, rtol=1e-13, atol=1e-300)
        # tippers (Tx, Ty) of post_process (fdfe_main.f90:705-708), written beside the
        # impedances, and the receiver E and H they and Z are formed from
        fld = S.receiver_fields(m, ex, quirks=q)
        for k, ff in enumerate(m.freq):
            _, tref, fref = O.post_process(om, ex[k, 0], ex[k, 1], ff, out_type, rd)
            assert np.abs(tref).max() > 0
            np.testing.assert_allclose(tip[k], tref, rtol=1e-12, atol=1e-14 * np.abs(tref).max())
            np.testing.assert_allclose(fld[k].reshape(-1, 10), fref, rtol=1e-13, atol=1e-15 * np.abs(fref).max())


def test_full_impedance_tensor():
    """out_type 3: the four components Z = E H^-1 of the two polarisations' receiver fields
    (post_process's E and H, fdfe_main.f90:600-700); Zxy and Zyx equal out_type 1's."""
    m = syn.small_aniso(freqs=(0.1, 10.0))
    rng = np.random.default_rng(1)
    ex = rng.standard_normal((2, 2, m.nl)) + 1j * rng.standard_normal((2, 2, m.nl))
    om = O.OracleModel(m.nx, m.ny, m.nz, m.nair, m.a, m.b, m.c, m.sigma, m.freq, m.recv)
    z4 = S.impedance(m, ex, out_type=3)
    z2 = S.impedance(m, ex, out_type=1)
    assert z4.shape == (m.nf, m.recv.shape[0], 8)
    np.testing.assert_allclose(z4[..., 2:6], z2, rtol=1e-14, atol=0)
    for k, ff in enumerate(m.freq):
        _, _, f = O.post_process(om, ex[k, 0], ex[k, 1], ff, 1, 2)
        E = np.stack([f[:, [0, 1]], f[:, [5, 6]]], axis=2)  # [rec][Ex, Ey][pol]
        H = np.stack([f[:, [2, 3]], f[:, [7, 8]]], axis=2)  # [rec][Hx, Hy][pol]
        Z = E @ np.linalg.inv(H)
        ref = np.stack([Z[:, 0, 0], Z[:, 0, 1], Z[:, 1, 0], Z[:, 1, 1]], 1)
        got = z4[k][:, 0::2] + 1j * z4[k][:, 1::2]
        np.testing.assert_allclose(got, ref, rtol=1e-11, atol=1e-13 * np.abs(ref).max())


def test_model_file_roundtrip(tmp_path):
    m = syn.small_aniso()
    name = str(tmp_path / "mod")
    m.write(name)
    r = S.Model.read(name)
    assert (r.nx, r.ny, r.nz, r.nair) == (m.nx, m.ny, m.nz, m.nair)
    np.testing.assert_array_equal(r.c, m.c)
    np.testing.assert_array_equal(r.sigma, m.sigma)
    np.testing.assert_array_equal(r.recv, m.recv)
    np.testing.assert_array_equal(r.freq, m.freq)


def test_reader_rejects_bad_level(tmp_path):
    m = syn.small_aniso()
    m.level = 2
    name = str(tmp_path / "bad")
    m.write(name)
    try:
        S.Model.read(name)
    except capi.SfdxError as e:
        assert e.code == 1
    else:
        raise AssertionError("level < 3 must be rejected (file_opt.f90:22-25)")


def test_ccv_and_res_files_use_the_reference_layout(tmp_path):
    """sfdx_write_ccv / sfdx_write_res: names and Fortran list-directed / Ew.d fields as
    solvers.f90:687-704 and file_opt.f90:131-158 write them."""
    import sfd_excmg_gb300 as S
    base = str(tmp_path / "m")
    S.write_ccv(base, 0.5, "xy", "excmg", 3, [1.0, 1.234e-3, 0.0, 9.996e-11])
    lines = open(base + "_0.50E+00_xy_excmg.ccv").read().splitlines()
    assert lines == ["           3", " 0.10E+01", " 0.12E-02", " 0.10E-09"]
    S.write_res(base, [10.0], np.array([[1.5, -2.0, 0.0]]), np.array([[[1.0, -0.25, 3.0e-4, 0.0]]]))
    fields = open(base + ".res").read().split()
    assert fields == ["0.15000E+01", "-0.20000E+01", "0.00000E+00", "0.10000E+02", "0", "0.10000E+01",
                      "-0.25000E+00", "0.30000E-03", "0.00000E+00"]
    # output_tipper: the tipper block follows the impedance block, row for row
    recv = np.array([[1.5, -2.0, 0.0], [2.5, 0.0, 0.0]])
    z = np.arange(16, dtype=float).reshape(2, 2, 4) + 1
    tip = -z / 100
    S.write_res(base, [10.0, 100.0], recv, z, tipper=tip)
    rows = [ln.split() for ln in open(base + ".res").read().splitlines()]
    assert len(rows) == 8
    for r, (k, i) in zip(rows, [(k, i) for k in range(2) for i in range(2)] * 2):
        assert [float(v) for v in r[:3]] == list(recv[i]) and float(r[3]) == [10.0, 100.0][k]
    np.testing.assert_allclose([[float(v) for v in r[5:]] for r in rows[:4]], z.reshape(4, 4), rtol=1e-5)
    np.testing.assert_allclose([[float(v) for v in r[5:]] for r in rows[4:]], tip.reshape(4, 4), rtol=1e-5)


def test_host_misfit_derivative_matches_finite_differences():
    """sfdx_impedance_misfit: the misfit equals the oracle's, and its derivative g
    (d misfit = 2 Re g^T dx) matches central differences in the real and imaginary
    parts of surface edge values, g = (d/dRe - i d/dIm) / 2."""
    import sfd_excmg_gb300 as S
    from oracle import oracle as O
    from sfd_excmg_gb300 import synthetic as syn
    m = syn.small_aniso(n=12, seed=2, freqs=(0.5,))
    om = O.OracleModel(m.nx, m.ny, m.nz, m.nair, m.a, m.b, m.c, m.sigma, m.freq, m.recv)
    u1, u2, _, _, _ = O.direct_solve(om, 0.5)
    ex = np.stack([u1, u2])[None]
    m2 = syn.small_aniso(n=12, seed=3, freqs=(0.5,))
    om2 = O.OracleModel(m.nx, m.ny, m.nz, m.nair, m.a, m.b, m.c, m2.sigma, m.freq, m.recv)
    v1, v2, _, _, _ = O.direct_solve(om2, 0.5)
    zobs = O.impedances(om2, np.stack([v1, v2])[None])
    phi, g = S.impedance_misfit(m, ex, zobs)
    assert abs(phi - O.misfit(om, zobs)) <= 1e-10 * phi
    nx, ny = m.nx, m.ny
    xnl = nx * (ny + 1) * (m.nz + 1)
    ynl = (nx + 1) * ny * (m.nz + 1)
    for p in (0, 1):
        # per orientation, the edge with the largest derivative (the receiver stencils
        # touch a few dozen surface edges)
        a = np.abs(g[0, p])
        edges = [int(np.argmax(a[:xnl])), xnl + int(np.argmax(a[xnl:xnl + ynl])),
                 xnl + ynl + int(np.argmax(a[xnl + ynl:]))]
        assert all(a[e] > 0 for e in edges)
        for e in edges:
            h = 1e-6 * np.abs(ex[0, p]).max()
            d = []
            for step in (h, 1j * h):
                xp = ex.copy()
                xm = ex.copy()
                xp[0, p, e] += step
                xm[0, p, e] -= step
                d.append((S.impedance_misfit(m, xp, zobs, grad=False)[0] -
                          S.impedance_misfit(m, xm, zobs, grad=False)[0]) / (2 * h))
            fd = (d[0] - 1j * d[1]) / 2
            assert abs(g[0, p, e] - fd) <= 1e-5 * abs(fd) + 1e-9 * np.abs(g).max(), (p, e, g[0, p, e], fd)


def _create(lib, opts, nx=16, ny=16, nz=16, nair=4, freqs=(1.0,)):
    """sfdx_plan_create on a small uniform mesh; returns (status, handle)."""
    dp = lambda v: np.ascontiguousarray(v, dtype=np.float64).ctypes.data_as(capi.c_double_p)  # noqa: E731
    a, b, c = np.full(nx, 50.0), np.full(ny, 50.0), np.full(nz, 50.0)
    f = np.asarray(freqs, dtype=np.float64)
    h = ctypes.c_void_p()
    st = lib.sfdx_plan_create(ctypes.byref(h), ctypes.byref(opts), nx, ny, nz, nair, dp(a), dp(b), dp(c), len(f), dp(f))
    return st, h.value


def test_plan_create_rejects_invalid_arguments_before_any_cuda_call(lib):
    """Every argument and option check of plan creation answers before the first CUDA
    call, so each invalid case returns its own status with no handle (also where no
    device exists)."""
    arg, mesh, unsup = 1, 2, 8
    cases = [
        (dict(ssor_omega=0.0), {}, arg),
        (dict(ssor_omega=2.0), {}, arg),
        (dict(ssor_omega=float("nan")), {}, arg),
        (dict(batch=1), {}, unsup),
        (dict(precond="I"), {}, unsup),  # ILU(0): a reference option that is not built
        (dict(precond="X"), {}, arg),
        (dict(solver=5), {}, arg),
        (dict(precision=2), {}, arg),
        (dict(excmg=1, level=2), {}, arg),
        (dict(div_cor=3), {}, arg),
        (dict(div_cor=2, corr_tol=0.0), {}, arg),
        (dict(eps=0.0), {}, arg),
        (dict(maxit_level=0), {}, arg),
        ({}, dict(nx=1), arg),
        ({}, dict(nair=17), arg),
        ({}, dict(freqs=(1.0, -2.0)), arg),
        ({}, dict(freqs=tuple(float(k + 1) for k in range(65))), unsup),  # 130 systems: above SFDX_MAX_SYSTEMS
        (dict(excmg=1, level=3), dict(nx=20), mesh),  # 20 cells do not split into 2^3 blocks
        (dict(excmg=1, level=4), dict(nx=8, ny=8, nz=8, nair=2), mesh),
    ]
    for kw, mesh_kw, want in cases:
        st, h = _create(lib, S.Opts.defaults(**kw), **mesh_kw)
        assert (st, h) == (want, None), (kw, mesh_kw, st)


def test_reader_rejects_truncated_and_malformed_files(tmp_path):
    """read_input on a cut-off or corrupted .fwd / .dat returns an error status (no
    read past the end, no partial model)."""
    m = syn.small_aniso()
    name = str(tmp_path / "mod")
    m.write(name)
    good = {ext: open(name + ext).read() for ext in (".fwd", ".dat")}
    cases = []
    for ext, txt in good.items():
        lines = txt.splitlines(keepends=True)
        for frac in (0.05, 0.3, 0.6, 0.95):
            # cut at the last whitespace before the point: whole tokens missing (a cut
            # inside a number can leave a shorter valid number, as in any reader)
            cut = txt[: int(len(txt) * frac)]
            cases.append((ext, cut[: max(cut.rfind(" "), cut.rfind("\n"), 0)]))
        cases.append((ext, "".join(lines[:-1])))              # last line missing
        cases.append((ext, ""))                                # empty file
        tok = txt.split()
        tok[len(tok) // 2] = "abc"                             # a non-number in the middle
        cases.append((ext, " ".join(tok)))
    for ext, bad in cases:
        for e2, t2 in good.items():
            open(name + e2, "w").write(bad if e2 == ext else t2)
        try:
            S.Model.read(name)
        except capi.SfdxError as e:
            assert e.code in (1, 7), (ext, len(bad), e.code)
        else:
            raise AssertionError(f"{ext} of {len(bad)} bytes accepted")


def test_sfd3d_host_reports_usage_and_input_errors(tmp_path):
    """The drop-in host `sfd3d <model> [level eps]` (sfd_excmg.f90:20-58): usage without
    a model name, an error status for missing or invalid model files, all before any
    device work."""
    import subprocess
    exe = os.path.join(os.path.dirname(capi.library_path()), "sfd3d")
    assert os.path.exists(exe), "sfd3d is built beside libsfdx.so"
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2 and "usage" in r.stderr
    r = subprocess.run([exe, str(tmp_path / "absent")], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "missing or malformed" in r.stderr, r.stderr
    m = syn.small_aniso()
    m.level = 2  # read_input rejects level < 3 (file_opt.f90:22-25)
    name = str(tmp_path / "lev2")
    m.write(name)
    r = subprocess.run([exe, name], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "invalid argument" in r.stderr, r.stderr
    assert not os.path.exists(name + ".res")


def test_opts_layout_agrees_across_c_header_fortran_shim_and_ctypes():
    """struct sfdx_opts has one layout in include/sfdx.h, the bind(c) type of the
    Fortran shim and the ctypes mirror: same fields, same order, same C types."""
    hdr = open(os.path.join(ROOT, "include", "sfdx.h")).read()
    body = re.search(r"typedef struct sfdx_opts \{(.*?)\} sfdx_opts;", hdr, re.S).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    c_fields = [(n, t) for t, n in re.findall(r"\b(int|double)\s+(\w+)\s*;", body)]
    f90 = open(os.path.join(ROOT, "sfd_excmg_gb300", "fortran", "sfdx_shim.f90")).read()
    ftype = re.search(r"type, bind\(c\) :: sfdx_opts(.*?)end type", f90, re.S).group(1)
    kind = {"integer(c_int)": "int", "real(c_double)": "double"}
    f_fields = [(n, kind[k]) for k, n in re.findall(r"(integer\(c_int\)|real\(c_double\))\s*::\s*(\w+)", ftype)]
    ct = {ctypes.c_int: "int", ctypes.c_double: "double"}
    py_fields = [(n, ct[t]) for n, t in capi.Opts._fields_]
    assert len(c_fields) >= 20
    assert f_fields == c_fields
    assert py_fields == c_fields


def test_reader_accepts_fortran_list_directed_forms(tmp_path):
    """The reference reads its inputs with list-directed read(unit,*): commas as
    separators, D exponents and r*c repeat counts read as the plain file does, and a
    value with trailing characters is an error."""
    m = syn.small_aniso()
    m.a[:] = 50.0
    name = str(tmp_path / "plain")
    m.write(name)
    r0 = S.Model.read(name)
    lines = open(name + ".fwd").read().splitlines(keepends=True)
    lines[1] = "%d, %s, %d, %d\n" % (m.level, ("%.6E" % m.eps).replace("E", "D"), m.solver, m.out_type)
    lines[3] = "%d*5.0D+01\n" % m.nx
    lines[7] = "6*0\n"
    alt = str(tmp_path / "listdir")
    open(alt + ".fwd", "w").write("".join(lines))
    open(alt + ".dat", "w").write(open(name + ".dat").read().replace(" ", ", "))
    r1 = S.Model.read(alt)
    assert (r1.level, r1.eps, r1.solver) == (r0.level, r0.eps, r0.solver)
    for f in ("a", "b", "c", "sigma", "freq", "recv"):
        np.testing.assert_array_equal(getattr(r1, f), getattr(r0, f), err_msg=f)
    lines[3] = "50.0x " * m.nx + "\n"
    open(alt + ".fwd", "w").write("".join(lines))
    try:
        S.Model.read(alt)
    except capi.SfdxError as e:
        assert e.code == 7
    else:
        raise AssertionError("a value with trailing characters must be rejected")


def test_reader_rejects_impossible_sizes(tmp_path):
    """Mesh, frequency and receiver counts are whole numbers in range: a negative,
    fractional or overflowing count is an input error, never an allocation size."""
    m = syn.small_aniso()
    name = str(tmp_path / "mod")
    m.write(name)
    fwd = open(name + ".fwd").read().splitlines(keepends=True)
    dat = open(name + ".dat").read().splitlines(keepends=True)
    nze = m.nz - m.nair
    bad_fwd = ["%d %d %d %d 0\n" % (-m.nx, m.ny, nze, m.nair), "%s %d %d %d 0\n" % ("16.5", m.ny, nze, m.nair),
               "%s %d %d %d 0\n" % ("1e30", m.ny, nze, m.nair), "%d %d %d %d 0\n" % (m.nx, m.ny, nze, -1)]
    for line in bad_fwd:
        open(name + ".fwd", "w").write("".join(fwd[:2] + [line] + fwd[3:]))
        try:
            S.Model.read(name)
        except capi.SfdxError as e:
            assert e.code == 7, (line, e.code)
        else:
            raise AssertionError(f"accepted mesh line {line!r}")
    open(name + ".fwd", "w").write("".join(fwd))
    open(name + ".dat", "w").write("".join(["0\n"] + dat[1 + m.nf:]))  # no frequencies
    try:
        S.Model.read(name)
    except capi.SfdxError as e:
        assert e.code == 7
    else:
        raise AssertionError("a model without frequencies was accepted")


def test_product_code_never_uses_the_oracle():
    """The oracle is test infrastructure: no module of the package imports it and no
    native source calls into it, so every product result comes from libsfdx."""
    import ast
    import glob
    pkg = os.path.join(ROOT, "sfd_excmg_gb300")
    for f in glob.glob(os.path.join(pkg, "**", "*.py"), recursive=True):
        tree = ast.parse(open(f).read())
        for n in ast.walk(tree):
            mods = []
            if isinstance(n, ast.Import):
                mods = [a.name for a in n.names]
            elif isinstance(n, ast.ImportFrom):
                mods = [n.module or ""]
            assert not any(m == "oracle" or m.startswith("oracle.") for m in mods), f
    for f in glob.glob(os.path.join(pkg, "**", "*.*"), recursive=True):
        if f.endswith((".cu", ".cuh", ".cpp", ".h", ".f90")):
            assert not re.search(r"\borc_\w+\s*\(|sfd_oracle", open(f).read()), f


def test_python_wrappers_check_array_sizes_before_calling_the_library():
    """Arrays handed to the C ABI are size-checked in Python: a wrong size raises
    ValueError before any native call (no read or write past a buffer)."""
    import pytest
    from sfd_excmg_gb300 import solver as sv
    m = syn.small_aniso()
    nx, ny, nz, nl = m.nx, m.ny, m.nz, m.nl
    x = np.zeros((nl, 2), complex)
    n0, n1 = sv._nl(nx // 4, ny // 4, nz // 4), sv._nl(nx // 2, ny // 2, nz // 2)
    bad = [
        lambda: S.apply_operator(nx, ny, nz, m.a, m.b, m.c, m.sigma, [1.0, 2.0], x[:-1]),
        lambda: S.apply_operator(nx, ny, nz, m.a[:-1], m.b, m.c, m.sigma, [1.0, 2.0], x),
        lambda: S.apply_operator(nx, ny, nz, m.a, m.b, m.c, m.sigma[:, :-1], [1.0, 2.0], x),
        lambda: S.precond_apply(nx, ny, nz, m.a, m.b, m.c, m.sigma, [1.0], np.zeros(nl + 1, complex)),
        lambda: S.krylov_solve(nx, ny, nz, m.a, m.b, m.c, m.sigma, [1.0, 1.0], x, x0=x[:10]),
        lambda: S.grad_correct(nx, ny, nz, m.a, m.b, m.c, m.sigma, [1.0, 1.0], x, x[:-2]),
        lambda: S.prolongate(nx, ny, nz, m.a, m.b, m.c, m.nair, np.zeros(n1, complex), np.zeros(n1, complex)),
        lambda: S.prolongate(nx + 2, ny, nz, m.a, m.b, m.c, m.nair, np.zeros(n0, complex), np.zeros(n1, complex)),
        lambda: S.build_rhs(nx, ny, nz, m.a, m.b, m.c, m.sigma, 1.0, np.zeros(nz, complex)),
        lambda: S.mesh_coarsen(m.a, m.b, m.c, m.sigma[:3], 1),
        lambda: S.mt1d(1.0, np.zeros((nz, 5)), m.c),
        lambda: S.impedance(m, np.zeros((m.nf, 1, nl), complex)),
        lambda: S.receiver_fields(m, np.zeros((m.nf, 2, nl - 1), complex)),
        lambda: S.impedance_misfit(m, np.zeros((m.nf, 2, nl), complex), np.zeros((m.nf, len(m.recv), 3))),
    ]
    for k, f in enumerate(bad):
        with pytest.raises(ValueError):
            f()
    # a malformed model is refused by Model.validate before a plan is created
    import copy
    for field, value in (("sigma", m.sigma[:, :-1]), ("a", m.a[:-1])):
        m2 = copy.deepcopy(m)
        setattr(m2, field, value)
        with pytest.raises(ValueError):
            S.Plan(m2)


def test_autograd_misfit_rejects_tensors_of_the_wrong_layout():
    """sigma_misfit takes sigma[6, ncell] and log_sigma_misfit log_sigma[ncell]: any
    other shape (for instance [ncell, 6]) is refused before the plan is touched."""
    import types
    import pytest
    torch = pytest.importorskip("torch")
    m = syn.small_aniso()
    fake_plan = types.SimpleNamespace(model=m)  # the check runs before any plan method
    zobs = np.zeros((m.nf, len(m.recv), 4))
    for bad in (torch.zeros(m.ncell, 6, dtype=torch.float64), torch.zeros(6, m.ncell - 1, dtype=torch.float64)):
        with pytest.raises(ValueError):
            S.sigma_misfit(bad, fake_plan, zobs)
    with pytest.raises(ValueError):
        S.log_sigma_misfit(torch.zeros(m.ncell + 1, dtype=torch.float64), fake_plan, zobs)


def test_topography_file_fills_the_air_cells_below_the_surface(tmp_path):
    """read_topo (file_opt.f90:97-128): for the columns n1..n2 x n1..n2, the n3 =
    int(height / c(nair+1)) air layers directly above the earth take sigma_hhs = 1e-2,
    written into components xx, xy and yz as the reference writes them."""
    m = syn.small_aniso()
    nx, ny, nair = m.nx, m.ny, m.nair
    cstep = m.c[nair]
    n1, n2 = 3, 6
    rng = np.random.default_rng(0)
    heights = cstep * np.array([0.0, 0.5, 1.0, 1.99, 2.0, 3.7, -1.0, 5.0] * 2)
    rng.shuffle(heights)
    m.topo = (n1, n2, heights)
    name = str(tmp_path / "topo")
    m.write(name)
    r = S.Model.read(name)
    expect = r.sigma.copy()
    expect[:, : nair * nx * ny] = 0
    expect[0:3, : nair * nx * ny] = 1e-9  # sigma_air in every air cell first
    q = 0
    for j in range(n1, n2 + 1):
        for i in range(n1, n2 + 1):
            n3 = int(heights[q] / cstep)
            q += 1
            for k in range(1, n3 + 1):
                cell = (nair - n3 + k - 1) * nx * ny + (j - 1) * nx + (i - 1)
                expect[[0, 3, 5], cell] = 1e-2
    np.testing.assert_array_equal(r.sigma, expect)
    assert (r.sigma[0, : nair * nx * ny] == 1e-2).sum() == sum(max(0, int(h / cstep)) for h in heights)


def test_noalloc_residual_refuses_misaligned_device_vectors(lib):
    """sfdx_residual_noalloc reads the caller's complex vectors as 16-byte values and
    sigma as doubles: misaligned pointers are refused with SFDX_ERR_ARG before any
    device work (the pointers below are never dereferenced)."""
    n = 8
    a = np.full(n, 10.0)
    f = np.array([1.0])
    rel = np.zeros(1)
    dp = lambda v: v.ctypes.data_as(capi.c_double_p)  # noqa: E731
    vp = ctypes.c_void_p
    cases = [(0x10000, 0x20008, 0x30000, 0x40000), (0x10000, 0x20000, 0x30004, 0x40000),
             (0x10000, 0x20000, 0x30000, 0x40008), (0x10004, 0x20000, 0x30000, 0x40000)]
    for sig, rhs, x, r in cases:
        st = lib.sfdx_residual_noalloc(n, n, n, dp(a), dp(a), dp(a), vp(sig), 1, dp(f), vp(rhs), vp(x), vp(r),
                                       dp(rel), None)
        assert st == 1, (hex(sig), hex(rhs), hex(x), hex(r), st)


def test_topography_receiver_planes_match_oracle():
    """sfdx_impedance_topo: receivers on each column's earth surface (the topo branch of
    post_process, fdfe_main.f90:604-616) in the reference form (plane one cell deep,
    vertical step c(nair+1)) and the corrected one, against the oracle; on flat ground the
    corrected form is the flat impedance."""
    m = syn.small_aniso(n=16, nair=8, freqs=(0.1, 10.0))
    rng = np.random.default_rng(3)
    ex = rng.standard_normal((2, 2, m.nl)) + 1j * rng.standard_normal((2, 2, m.nl))
    om = O.OracleModel(m.nx, m.ny, m.nz, m.nair, m.a, m.b, m.c, m.sigma, m.freq, m.recv)
    abr = np.array([3, 14, 2, 15, 2, 12], np.int32)
    cols = (abr[1] - abr[0] + 1) * (abr[3] - abr[2] + 1)
    topo = rng.uniform(0.0, 0.8 * m.c[:m.nair].sum(), cols)
    for q, corrected in ((capi.QUIRKS_REFERENCE, False), (capi.QUIRKS_REFERENCE & ~capi.QUIRK_TOPO_PLANE, True)):
        got = S.impedance_topo(m, ex, abr, topo, quirks=q)
        mcol, czcol = O.receiver_planes(om, abr, topo, corrected=corrected)
        assert len(set(mcol.tolist())) > 2  # the planes follow the surface
        for k, ff in enumerate(m.freq):
            ref, _, _ = O.post_process_topo(om, ex[k, 0], ex[k, 1], ff, mcol, czcol, 1, 2)
            np.testing.assert_allclose(got[k], ref, rtol=1e-12, atol=1e-14 * np.abs(ref).max())
    flat = S.impedance_topo(m, ex, abr, np.zeros(cols), quirks=capi.QUIRKS_REFERENCE & ~capi.QUIRK_TOPO_PLANE)
    np.testing.assert_allclose(flat, S.impedance(m, ex), rtol=1e-14, atol=0)
