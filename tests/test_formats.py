"""File formats on either side of the path (include/gbattract_io.h), pinned to
the reference's own readers and writers compiled in oracle/_ref.

Every comparison with the reference is exact: bitwise for parsed numbers,
byte-for-byte for written files.  Synthetic files live in tmp_path; where the
reference tree oracle/_ref was built from is present, its own test resources
(reduced PDBs, attract.par, alphabet, DOF and score files) are read by both
sides as well.  Round trips through this library's own reader and writer run
everywhere."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def fmt(pkg):
    from gbattract import formats
    return formats


@pytest.fixture(scope="module")
def ref(oracle):
    if not oracle.ref_available():
        pytest.skip("reference CPU path not built on this host")
    return oracle


@pytest.fixture(scope="module")
def resources(oracle):
    root = oracle.ref_root()
    if root is None or not (root / "test" / "resources").is_dir():
        pytest.skip("reference test resources not present on this host")
    return root / "test" / "resources"


def pdb_line(i, x, y, z, t, q):
    return f"ATOM  {i:5d} CA   ALA A{i:4d}    {x:8.3f}{y:8.3f}{z:8.3f}{t:5d}{q:8.3f} 0 1.00\n"


def write_pdb(path, xyz, t, q, terminate=True, blank_every=0):
    lines = []
    for i in range(len(t)):
        lines.append(pdb_line(i + 1, *xyz[:, i], int(t[i]), q[i]))
        if blank_every and i % blank_every == blank_every - 1:
            lines.append("\n")
    s = "".join(lines)
    path.write_text(s if terminate else s.rstrip("\n"))


# ---------------------------------------------------------------- PDB --

def test_pdb_matches_reference_reader(fmt, ref, tmp_path):
    rng = np.random.default_rng(3)
    n = 57
    xyz = rng.uniform(-80, 80, (3, n))
    t = rng.integers(1, 33, n)
    t[5] = 99
    q = rng.choice([0.0, 1.0, -1.0, 0.5], n)
    for terminate in (True, False):
        p = tmp_path / f"p{int(terminate)}.pdb"
        write_pdb(p, xyz, t, q, terminate=terminate, blank_every=7)
        got = fmt.read_pdb(p)
        want = ref.ref_read_pdb(p, default_map=False)
        for a, b in zip(got, want):
            assert np.array_equal(a, b)
        # an unterminated last line is dropped, as the reference does
        assert got[1].shape[0] == (n if terminate else n - 1)


def test_pdb_reference_resources(fmt, ref, resources):
    for name in ("receptorr.pdb", "ligandr.pdb"):
        got = fmt.read_pdb(resources / name)
        want = ref.ref_read_pdb(resources / name, default_map=False)
        assert got[1].shape[0] > 100
        for a, b in zip(got, want):
            assert np.array_equal(a, b)


def test_pdb_short_line_is_an_error(fmt, tmp_path):
    p = tmp_path / "bad.pdb"
    p.write_text(pdb_line(1, 1, 2, 3, 4, 0.0) + "END\n")
    with pytest.raises(fmt.IoError):
        fmt.read_pdb(p)


# ------------------------------------------------------------ params --

def write_par(path, shape, T, rng):
    r = rng.uniform(2.5, 5.0, (T, T))
    e = rng.uniform(0.05, 9.0, (T, T))
    e[0, 1] = 0.0                        # rc = ac = 0 -> emin = rmin2 = 0
    ip = rng.integers(-1, 2, (T, T))
    with open(path, "w") as f:
        f.write(f"{shape} {T} 0.0 0.0\n")
        for m, fmtc in ((r, "{:.6f}"), (e, "{:.6f}"), (ip, "{:d}")):
            for i in range(T):
                f.write(" ".join(fmtc.format(v) for v in m[i]) + "\n")


@pytest.mark.parametrize("shape", [8, 12])
def test_params_match_reference_reader(fmt, ref, tmp_path, shape):
    p = tmp_path / f"a{shape}.par"
    write_par(p, shape, 7, np.random.default_rng(shape))
    got = fmt.read_params(p)
    tab, ps = ref.ref_read_params(p)
    assert got.potshape == ps
    assert got.table.tobytes() == tab.tobytes()


def test_params_reference_resource(fmt, ref, resources):
    got = fmt.read_params(resources / "attract.par")
    tab, ps = ref.ref_read_params(resources / "attract.par")
    assert got.num_types == 98 and got.potshape == ps
    assert got.table.tobytes() == tab.tobytes()


def test_params_bad_shape(fmt, tmp_path):
    p = tmp_path / "bad.par"
    p.write_text("9 1 0 0\n1\n1\n1\n")
    with pytest.raises(fmt.IoError, match="potential shape"):
        fmt.read_params(p)


# ------------------------------------------------- alphabet and types --

def test_type_mapping_matches_configurator(fmt, ref, tmp_path):
    p = tmp_path / "grid.alphabet"
    alpha = [2, 5, 7, 11, 13, 99, 20]
    p.write_text("".join(f"{a}\n" for a in alpha))
    assert list(fmt.read_alphabet(p)) == alpha
    types = np.array([0, 2, 5, 99, 20, 11, 13, 7, 2], np.uint32)
    t, m = fmt.map_types(alpha, types)
    rt, rm, ra = ref.ref_map_types(p, types)
    assert list(ra) == alpha
    assert np.array_equal(t, rt) and np.array_equal(m, rm)
    assert list(m) == [0, 1, 2, 0, 7, 4, 5, 3, 1]
    with pytest.raises(fmt.IoError, match="not in the grid alphabet"):
        fmt.map_types(alpha, np.array([3], np.uint32))


def test_alphabet_reference_resource(fmt, ref, resources, pkg):
    lig = fmt.read_pdb(resources / "ligandr.pdb")
    alpha = fmt.read_alphabet(resources / "receptorgrid.alphabet")
    t, m = fmt.map_types(alpha, lig[1])
    rt, rm, ra = ref.ref_map_types(resources / "receptorgrid.alphabet", lig[1])
    assert np.array_equal(alpha, ra) and np.array_equal(t, rt) and np.array_equal(m, rm)


# -------------------------------------------------------------- DOFs --

def synth_dof(fmt, S=9, modes=(0, 0), seed=1, auto=False):
    rng = np.random.default_rng(seed)
    vals = np.zeros((S, 2, 16), np.float32)
    cnt = np.zeros((S, 2), np.int32)
    vals[:, 1, :3] = rng.uniform(-np.pi, np.pi, (S, 3))
    vals[:, 1, 3:6] = rng.uniform(-50, 50, (S, 3))
    vals[:, 0, :6] = 0
    vals[1, 0, :6] = [0.3, -0.2, 1.1, 2.5, -1.0, 0.75]   # a moved receptor
    for m, k in enumerate(modes):
        vals[:, m, 6:6 + k] = rng.uniform(-1, 1, (S, k))
        cnt[:, m] = 6 + k
    piv = [] if auto else [(32.823, -6.395, 23.484), (51.143, 7.680, 38.110)]
    return fmt.DofFile(vals, cnt, auto_pivot=auto, centered_receptor=False,
                       centered_ligands=True, pivots=piv)


@pytest.mark.parametrize("auto,modes", [(False, (0, 0)), (True, (3, 5))])
def test_dof_write_read_matches_reference(fmt, ref, tmp_path, auto, modes):
    d = synth_dof(fmt, modes=modes, auto=auto)
    p = tmp_path / "poses.dat"
    fmt.write_dof(p, d, energies=np.linspace(-5, 1, d.num_structures))
    back = fmt.read_dof(p)
    assert np.array_equal(back.values, d.values) and np.array_equal(back.counts, d.counts)
    assert back.auto_pivot == auto and back.centered_ligands and not back.centered_receptor
    assert np.array_equal(np.asarray(back.pivots, np.float32).reshape(-1, 3),
                          np.asarray(d.pivots, np.float32).reshape(-1, 3))
    vals, cnt, h = ref.ref_read_dof(p)
    assert np.array_equal(vals, back.values) and np.array_equal(cnt, back.counts)
    assert h["auto_pivot"] == auto and h["centered_ligands"] and not h["centered_receptor"]
    assert np.array_equal(np.asarray(h["pivots"], np.float32).reshape(-1, 3),
                          np.asarray(back.pivots, np.float32).reshape(-1, 3))


def test_dof_reference_resources(fmt, ref, resources):
    for name in ("systsearch.dat", "out_docking_orig.dat", "readDof_test.dat"):
        got = fmt.read_dof(resources / name)
        vals, cnt, h = ref.ref_read_dof(resources / name)
        assert got.num_structures > 0
        assert np.array_equal(got.values, vals) and np.array_equal(got.counts, cnt)
        assert got.auto_pivot == h["auto_pivot"]
        assert np.array_equal(np.asarray(got.pivots, np.float32).reshape(-1, 3),
                              np.asarray(h["pivots"], np.float32).reshape(-1, 3))


def test_dof_incomplete_structure_is_an_error(fmt, tmp_path):
    p = tmp_path / "bad.dat"
    p.write_text("#pivot auto\n#centered receptor: false\n#centered ligands: false\n#1\n"
                 "0 0 0 0 0 0\n1 2 3 4 5 6\n#2\n0 0 0 0 0 0\n")
    with pytest.raises(fmt.IoError, match="incomplete"):
        fmt.read_dof(p)


# ------------------------------------------------------------ frames --

def test_auto_pivot_and_glob2rec_match_reference(fmt, ref):
    rng = np.random.default_rng(11)
    xyz = rng.normal(20, 15, (3, 333)).astype(np.float32)
    assert np.array_equal(fmt.auto_pivot(xyz), ref.ref_auto_pivot(xyz))
    n = 400
    rec = np.zeros((n, 6), np.float32)
    lig = np.zeros((n, 6), np.float32)
    lig[:, :3] = rng.uniform(-60, 60, (n, 3))
    lig[:, 3:] = rng.uniform(-np.pi, np.pi, (n, 3))
    rec[n // 2:, :3] = rng.uniform(-5, 5, (n - n // 2, 3))
    rec[n // 4:, 3:] = rng.uniform(-np.pi, np.pi, (n - n // 4, 3))
    # gimbal-lock branches of rotmat2euler: receptor and ligand rotations that cancel
    rec[-20:, 3:] = lig[-20:, 3:]
    rec[-10:, 3:] = 0.0
    lig[-10:, 3:] = 0.0
    rec[-10:, 4] = 0.4
    lig[-10:, 4] = 0.4
    pr = np.array([3.5, -2.25, 7.0], np.float32)
    pl = np.array([-1.0, 4.0, 0.5], np.float32)
    for crec in (False, True):
        for clig in (False, True):
            a = fmt.glob2rec(rec, lig, pr, pl, crec, clig)
            b = ref.ref_glob2rec(rec, lig, pr, pl, crec, clig)
            assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert np.all(a[0] == 0)


def test_glob2rec_modes_stride(fmt):
    rng = np.random.default_rng(2)
    rec = np.zeros((5, 26), np.float32)
    lig = rng.uniform(-1, 1, (5, 26)).astype(np.float32)
    rec[:, 6:] = 7.0
    a6 = fmt.glob2rec(rec[:, :6], lig[:, :6], [1, 2, 3], [0, 0, 0], False, False)
    a = fmt.glob2rec(rec, lig, [1, 2, 3], [0, 0, 0], False, False)
    assert np.array_equal(a[1][:, :6], a6[1]) and np.array_equal(a[1][:, 6:], lig[:, 6:])
    assert np.all(a[0][:, 6:] == 7.0)


# ----------------------------------------------------------- results --

def test_result_stream_bytes_match_reference(fmt, ref, tmp_path):
    rng = np.random.default_rng(5)
    r = rng.normal(0, 50, (17, 7)).astype(np.float32)
    r[0] = 0.0
    r[1, 0] = -1.5e-7
    fmt.write_results(tmp_path / "a.txt", r)
    ref.ref_write_results(tmp_path / "b.txt", r)
    assert (tmp_path / "a.txt").read_bytes() == (tmp_path / "b.txt").read_bytes()
    rm = rng.normal(0, 5, (6, 27)).astype(np.float32)
    fmt.write_results(tmp_path / "c.txt", rm, n_modes_rec=3, n_modes_lig=4)
    ref.ref_write_results(tmp_path / "d.txt", rm, 3, 4)
    assert (tmp_path / "c.txt").read_bytes() == (tmp_path / "d.txt").read_bytes()


@pytest.mark.parametrize("style,modes", [(0, (0, 0)), (1, (0, 0)), (1, (3, 2))])
def test_results_read_back_like_reference(fmt, ref, tmp_path, style, modes):
    rng = np.random.default_rng(9)
    width = 7 if modes == (0, 0) else 27
    r = rng.normal(0, 20, (11, width)).astype(np.float32)
    p = tmp_path / "r.score"
    fmt.write_results(p, r, *modes, style=style)
    fmt.write_results(p, r[:2], *modes, style=style, append=True)
    got = fmt.read_results(p)
    want = ref.ref_read_results(p)
    assert len(got) == len(want) == 13
    for a, b in zip(got, want):
        assert np.array_equal(a, b)
    # energies and the ligand gradients survive the text form
    rows = np.concatenate([r, r[:2]])
    for i, rec in enumerate(got):
        assert rec[0] == pytest.approx(float(rows[i, 0]), rel=1e-7, abs=1e-30)
        if style == 0:
            lig = rec[1:7]
        else:
            lig = rec[7 + modes[0]:13 + modes[0]]
        assert np.allclose(lig, np.concatenate([rows[i, 4:7], rows[i, 1:4]]), rtol=1e-7, atol=0)


def test_results_reference_score_resource(fmt, ref, resources):
    p = resources / "out_attract_modes_no_fixRec.score"
    got = fmt.read_results(p)
    want = ref.ref_read_results(p)
    assert len(got) == len(want) > 0
    for a, b in zip(got, want):
        assert np.array_equal(a, b)


def test_modes_stream_form_is_rejected_by_reader(fmt, tmp_path):
    rm = np.ones((2, 27), np.float32)
    p = tmp_path / "m.txt"
    fmt.write_results(p, rm, n_modes_rec=1, n_modes_lig=1)
    with pytest.raises(fmt.IoError, match="not part of a result record"):
        fmt.read_results(p)


# -------------------------------------------------------------- grids --

@pytest.fixture(scope="module")
def small_grid(pkg, oracle):
    """A 60-bead receptor, a 5-type alphabet and a tight box (a few MB of file)."""
    import dataclasses
    wl = pkg.synth.make_pair(5, 60, 25, 16, (13.0, 18.0), seed=21)
    alphabet = [2, 3, 5, 7, 11]
    rng = np.random.default_rng(4)
    rt = rng.choice(alphabet, wl.rec.n).astype(np.uint32)
    lt = rng.choice(alphabet, wl.lig.n).astype(np.uint32)
    chan = {t: c + 1 for c, t in enumerate(alphabet)}
    rec = pkg.Protein(xyz=wl.rec.xyz, type=rt, mapped=np.zeros_like(rt), charge=wl.rec.charge)
    lig = pkg.Protein(xyz=wl.lig.xyz, type=lt, mapped=np.array([chan[t] for t in lt], np.uint32),
                      charge=wl.lig.charge)
    wl = dataclasses.replace(wl, rec=rec, lig=lig)
    opts = pkg.GridOptions(alphabet=alphabet, margin=4.0, outer_ext=8)
    grid = oracle.build_grid(wl.rec, wl.params, opts)
    return wl, grid, opts


def test_grid_file_bytes_match_reference_writer(fmt, ref, small_grid, tmp_path):
    wl, grid, opts = small_grid
    info = fmt.grid_header(grid, opts.alphabet, wl.rec.n, pivot=(1.5, -2.0, 0.25),
                           gridextension=opts.outer_ext)
    fmt.write_grid(tmp_path / "a.grid", grid, opts.alphabet, info, rec_xyz=wl.rec.xyz)
    ref.ref_write_grid_file(tmp_path / "b.grid", grid, opts.alphabet, info, rec_xyz=wl.rec.xyz)
    a, b = (tmp_path / "a.grid").read_bytes(), (tmp_path / "b.grid").read_bytes()
    assert len(a) == len(b) and a == b


def test_grid_file_reads_back_like_reference(fmt, ref, small_grid, tmp_path, oracle):
    wl, grid, opts = small_grid
    info = fmt.grid_header(grid, opts.alphabet, wl.rec.n, gridextension=opts.outer_ext)
    p = tmp_path / "g.grid"
    fmt.write_grid(p, grid, opts.alphabet, info)
    back, info2 = fmt.read_grid(p)
    ci, inner, co, outer, cn, nlg, nll, dp2 = ref.ref_read_grid_file(p, info2)
    # identical to the reference reader ...
    assert np.array_equal(back.inner_data, inner) and np.array_equal(back.outer_data, outer)
    assert np.array_equal(back.nl_list, nll)
    occupied = back.nl_grid[..., 0] > 0
    assert np.array_equal(back.nl_grid[..., 0], nlg[..., 0])
    assert np.array_equal(back.nl_grid[..., 1], nlg[..., 1])
    for d, c in ((back.inner, ci), (back.outer, co)):
        assert d.numGrids == c.numGrids and tuple(d.dimN) == tuple(c.dimN)
        assert np.float32(d.gridSpacing) == np.float32(c.gridSpacing)
        assert np.array_equal(np.float32(d.posMin), np.float32(tuple(c.posMin)))
    assert np.float32(back.nl.dPlateau) ** 2 == np.float32(dp2)
    # ... and to the grid that was written (channels in ascending type order)
    assert np.array_equal(back.inner_data, grid.inner_data)
    assert np.array_equal(back.outer_data, grid.outer_data)
    assert np.array_equal(back.nl_list, grid.nl_list)
    assert np.array_equal(back.nl_grid[occupied], grid.nl_grid[occupied])
    for d, g in ((back.inner, grid.inner), (back.outer, grid.outer)):
        assert np.array_equal(np.float32(d.posMin), np.float32(g.posMin))
        assert tuple(d.dimN) == tuple(g.dimN) and np.float32(d.gridSpacing) == np.float32(g.gridSpacing)
    # scoring on the read-back grid equals scoring on the original
    e0 = oracle.energy_6d(wl.rec, wl.lig, grid, wl.params, wl.dofs)
    e1 = oracle.energy_6d(wl.rec, wl.lig, back, wl.params, wl.dofs)
    assert np.array_equal(e0, e1)


def test_grid_writer_rejects_non_attract_layout(fmt, small_grid, tmp_path):
    wl, grid, opts = small_grid
    info = fmt.grid_header(grid, opts.alphabet, wl.rec.n, gridextension=opts.outer_ext + 2)
    with pytest.raises(fmt.IoError, match="outer origin"):
        fmt.write_grid(tmp_path / "x.grid", grid, opts.alphabet, info)


def test_load_docking_inputs_like_configurator(fmt, ref, pkg, tmp_path, small_grid, oracle):
    """The configurator-style loader on a full file set: proteins, parameters,
    alphabet mapping, pivots, receptor-frame DOFs and the -pivot grid shift
    agree with the reference's own routines, and scoring the loaded run
    reproduces scoring the original in-memory pair."""
    wl, grid, opts = small_grid
    rng = np.random.default_rng(12)
    shift_r = np.array([12.5, -3.25, 40.0], np.float32)
    shift_l = np.array([-7.0, 22.0, 5.5], np.float32)
    # files in the absolute frame: beads moved by a pivot, grid moved with them
    rxyz = (wl.rec.xyz + shift_r[:, None]).astype(np.float32)
    lxyz = (wl.lig.xyz + shift_l[:, None]).astype(np.float32)
    write_pdb(tmp_path / "rec.pdb", rxyz, wl.rec.type, wl.rec.charge)
    write_pdb(tmp_path / "lig.pdb", lxyz, wl.lig.type, wl.lig.charge)
    (tmp_path / "grid.alphabet").write_text("".join(f"{a}\n" for a in opts.alphabet))
    write_par(tmp_path / "attract.par", 8, 32, rng)
    rec_abs = pkg.Protein(xyz=rxyz, type=wl.rec.type, mapped=wl.rec.mapped, charge=wl.rec.charge)
    gabs = oracle.build_grid(rec_abs, wl.params, opts)
    info = fmt.grid_header(gabs, opts.alphabet, wl.rec.n, pivot=shift_r, gridextension=opts.outer_ext)
    fmt.write_grid(tmp_path / "rec.grid", gabs, opts.alphabet, info)
    S = 6
    vals = np.zeros((S, 2, 16), np.float32)
    cnt = np.full((S, 2), 6, np.int32)
    vals[:, 1, :3] = rng.uniform(-3, 3, (S, 3))
    vals[:, 1, 3:6] = rng.uniform(-30, 30, (S, 3))
    d = fmt.DofFile(vals, cnt, auto_pivot=True, centered_receptor=False, centered_ligands=False)
    fmt.write_dof(tmp_path / "poses.dat", d)
    run = fmt.load_docking_inputs(tmp_path / "poses.dat", tmp_path / "rec.pdb", tmp_path / "lig.pdb",
                                  tmp_path / "attract.par", tmp_path / "rec.grid",
                                  tmp_path / "grid.alphabet")
    rfile = ref.ref_read_pdb(tmp_path / "rec.pdb", default_map=False)[0]   # %8.3f columns
    lfile = ref.ref_read_pdb(tmp_path / "lig.pdb", default_map=False)[0]
    pr, pl = ref.ref_auto_pivot(rfile), ref.ref_auto_pivot(lfile)
    assert np.array_equal(run.pivots[0], pr) and np.array_equal(run.pivots[1], pl)
    assert np.array_equal(run.rec.xyz, (rfile - pr[:, None]).astype(np.float32))
    _, lm, _ = ref.ref_map_types(tmp_path / "grid.alphabet", wl.lig.type)
    assert np.array_equal(run.lig.mapped, lm) and np.array_equal(run.lig.mapped, wl.lig.mapped)
    _, want = ref.ref_glob2rec(d.dofs6(0), d.dofs6(1), pr, pl, False, False)
    assert np.array_equal(run.dofs, want)
    tab, _ = ref.ref_read_params(tmp_path / "attract.par")
    assert run.params.table.tobytes() == tab.tobytes()
    # the grid is shifted into the pivotized receptor frame (GridUnion::translate)
    want_grid = fmt.translate_grid(gabs, -pr)
    for got_d, want_d in ((run.grid.inner, want_grid.inner), (run.grid.outer, want_grid.outer),
                          (run.grid.nl, want_grid.nl)):
        assert np.array_equal(np.float32(got_d.posMin), np.float32(want_d.posMin))
    assert np.array_equal(run.grid.inner_data, gabs.inner_data)
    assert np.array_equal(run.grid.nl_list, gabs.nl_list)
    e = oracle.energy_6d(run.rec, run.lig, run.grid, run.params, run.dofs)
    assert np.all(np.isfinite(e))
