"""GPU converters and kernels of every format except CSR, through the C ABI.

Converters: the exported arrays (reference layout) must be bit-identical to
the reference's own converter output (golden fixture digests) and to the
oracle restatement on larger seeded matrices.
SpMV / SpMM: per-row bound |y_i - y_ref_i| <= 8*nnz_i*eps*|alpha|*sum_j|a_ij
x_j| + 2*eps*|beta*y0_i| against the FP64 CSR result (y_ref) on the same
inputs, FP64 and FP32."""
import numpy as np
import pytest

from golden_util import ALPHA, BETA, digest, files, load
from gpu_util import to_dev, to_host
from oracle import tolerance_ok

pytestmark = pytest.mark.gpu

CASES = files()


def gpu_convert(L, M, fn, kw):
    """Runs the library converter named like the oracle's, mapping its kwargs."""
    if fn == "csr_to_ell":
        return L.csr_to_ell(M, kw.get("ld", 0))
    if fn == "csr_to_sell":
        return L.csr_to_sell(M, kw.get("C_", 0), kw.get("align", 0) or 0)
    if fn == "csr_to_sell_c_sigma":
        return L.csr_to_sell_c_sigma(M, kw.get("sigma", 0), kw.get("C_", 0), kw.get("align", 0) or 0)
    if fn == "csr_to_sell_c_R":
        return L.csr_to_sell_c_R(M, kw.get("C_", 0), kw.get("align", 0) or 0)
    if fn == "csr_to_dia" and hasattr(L, "csr_to_dia"):
        return L.csr_to_dia(M, kw.get("max_diags", 0), kw.get("align", 0) or 0)
    if fn == "csr_to_bsr" and hasattr(L, "csr_to_bsr"):
        return L.csr_to_bsr(M, kw.get("r", 0), kw.get("c", 0) or 0)
    if fn == "csr_to_csr5" and hasattr(L, "csr_to_csr5"):
        return L.csr_to_csr5(M)
    return None


@pytest.mark.parametrize("path", CASES, ids=[p.stem for p in CASES])
def test_converters_match_reference(path):
    from sspmv_gb300 import lespmv as L
    z, meta, A = load(path)
    M = L.csr_from_host(A)
    checked = 0
    for key, rec in meta["conv"].items():
        G = gpu_convert(L, M, rec["fn"], rec["kw"])
        if G is None:
            continue
        out = G.export()
        for name, d in rec["digests"].items():
            assert name in out, (key, name)
            assert list(out[name].shape) == rec["shapes"][name], (key, name, out[name].shape)
            assert digest(out[name]) == d, f"{path.stem}:{key}:{name} differs from the reference"
        for name, v in rec["scalars"].items():
            if name in out:
                assert int(out[name]) == v, (key, name)
        checked += 1
    assert checked >= 9


SPMV_FORMATS = [("ell", "csr_to_ell", {}), ("sell", "csr_to_sell", {}), ("sell_c_sigma", "csr_to_sell_c_sigma", {}),
                ("sell_c_R", "csr_to_sell_c_R", {}), ("dia", "csr_to_dia", {}), ("bsr", "csr_to_bsr", {}),
                ("coo", "csr_to_coo", {}), ("csr5", "csr_to_csr5", {})]


@pytest.mark.parametrize("path", CASES, ids=[p.stem for p in CASES])
def test_spmv_golden(path, oracle_lib):
    from sspmv_gb300 import lespmv as L
    z, meta, A = load(path)
    dt = A.values.dtype
    x, y0 = z["x"], z["y0"]
    y64, absum = oracle_lib.spmm_ref(A, x, ALPHA, BETA, y0)
    nnz_row = np.diff(A.row_offset)
    has_dups = "in_coo_row" in z.files
    M = L.csr_from_host(A)
    for fmt, fn, kw in SPMV_FORMATS:
        conv = getattr(L, fn, None)
        if conv is None:
            continue
        try:
            G = conv(M, **kw)
        except L.SSPMVError as e:
            assert e.status == 2 and fmt == "dia", (fmt, e)  # DIA over max_diags
            continue
        y = to_dev(y0)
        L.LeSpMV(ALPHA, G, to_dev(x), BETA, y)
        yg = to_host(y)
        if has_dups and fmt in ("dia", "bsr"):
            yr = z.get(f"y_{fmt}_1")  # duplicates overwrite: compare with the reference itself
            assert oracle_lib.max_rel_error(yg, yr) < 5 * np.sqrt(np.finfo(dt).eps), fmt
            continue
        ok, mx, med = tolerance_ok(yg, y64, absum, nnz_row, dt, ALPHA, BETA, y0)
        assert ok, f"{fmt}: max normalised error {mx}"


FAMILIES = {
    "powerlaw": lambda s: s.powerlaw(30000, 1.8, 16.0, 3000, 0.02),
    "uniform": lambda s: s.uniform(20000, 32, 0.01),
    "banded": lambda s: s.banded(30000),
    "block": lambda s: s.block(20000, 4, 4000),
    "wide": lambda s: s.uniform(5000, 12, 0.05, num_cols=17000),
}

ORACLE_CONV = {
    "ell": lambda O, A: O.csr_to_ell(A, 0),
    "sell": lambda O, A: O.csr_to_sell(A, 8, 4),
    "sell_c_sigma": lambda O, A: O.csr_to_sell_c_sigma(A, 256, 32, 1),
    "sell_c_R": lambda O, A: O.csr_to_sell_c_R(A, 16),
    "coo": lambda O, A: O.csr_to_coo(A),
    "dia": lambda O, A: O.csr_to_dia(A),
    "bsr4x4": lambda O, A: O.csr_to_bsr(A, 4, 4),
    "bsr2x8": lambda O, A: O.csr_to_bsr(A, 2, 8),
    "bsr3x5": lambda O, A: O.csr_to_bsr(A, 3, 5),
    "csr5": lambda O, A: O.csr_to_csr5(A),
    "csr5_w32": lambda O, A: O.csr_to_csr5(A, 16, 32),
    "csr5_s12_w4": lambda O, A: O.csr_to_csr5(A, 12, 4),
    "sell_c4": lambda O, A: O.csr_to_sell(A, 4, 4),
    "scs_c8": lambda O, A: O.csr_to_sell_c_sigma(A, 256, 8, 1),
    "scr_c16": lambda O, A: O.csr_to_sell_c_R(A, 16),
}


GPU_CONV = {
    "ell": lambda L, M: L.csr_to_ell(M, 0),
    "sell": lambda L, M: L.csr_to_sell(M, 8, 4),
    "sell_c_sigma": lambda L, M: L.csr_to_sell_c_sigma(M, 256, 32, 1),
    "sell_c_R": lambda L, M: L.csr_to_sell_c_R(M, 16),
    "coo": lambda L, M: L.csr_to_coo(M),
    "dia": lambda L, M: L.csr_to_dia(M),
    "bsr4x4": lambda L, M: L.csr_to_bsr(M, 4, 4),
    "bsr2x8": lambda L, M: L.csr_to_bsr(M, 2, 8),
    "bsr3x5": lambda L, M: L.csr_to_bsr(M, 3, 5),
    "csr5": lambda L, M: L.csr_to_csr5(M),
    "csr5_w32": lambda L, M: L.csr_to_csr5(M, 16, 32),
    "csr5_s12_w4": lambda L, M: L.csr_to_csr5(M, 12, 4),
    # narrow chunks: long rows in the compact overflow path
    "sell_c4": lambda L, M: L.csr_to_sell(M, 4, 4),
    "scs_c8": lambda L, M: L.csr_to_sell_c_sigma(M, 256, 8, 1),
    "scr_c16": lambda L, M: L.csr_to_sell_c_R(M, 16),
}


@pytest.mark.parametrize("dt", [np.float64, np.float32], ids=["f64", "f32"])
@pytest.mark.parametrize("fam", list(FAMILIES))
def test_families_convert_and_spmm(fam, dt, oracle_lib):
    from sspmv_gb300 import lespmv as L
    from sspmv_gb300 import synth
    A = synth.generate(FAMILIES[fam](synth), 3, dt)
    M = L.csr_from_host(A)
    nnz_row = np.diff(A.row_offset)
    for fmt in GPU_CONV:
        if fmt == "ell" and fam == "powerlaw":
            continue
        if fmt.startswith("bsr") and fam in ("powerlaw", "uniform", "wide"):
            continue  # block fill explodes on scattered columns
        ref = ORACLE_CONV[fmt](oracle_lib, A)
        if ref is None:  # DIA over max_diags
            with pytest.raises(L.SSPMVError) as e:
                GPU_CONV[fmt](L, M)
            assert e.value.status == 2
            continue
        G = GPU_CONV[fmt](L, M)
        out = G.export()
        for name, arr in ref.items():
            if isinstance(arr, np.ndarray):
                assert np.array_equal(out[name].view(np.uint8), arr.view(np.uint8)), (fam, fmt, name)
        for k in (1, 3, 8):
            X = synth.vector(A.num_cols, 0, dt, k).reshape(A.num_cols, k)
            Y0 = synth.vector(A.num_rows, 9, dt, k).reshape(A.num_rows, k)
            Y = to_dev(Y0)
            L.spmm(ALPHA, G, to_dev(X), BETA, Y)
            y64, absum = oracle_lib.spmm_ref(A, X, ALPHA, BETA, Y0)
            ok, mx, _ = tolerance_ok(to_host(Y), y64, absum, nnz_row, dt, ALPHA, BETA, Y0)
            assert ok, f"{fam}/{fmt}/k={k}: max normalised error {mx}"


def test_sigma_not_multiple_of_c_is_rejected():
    from sspmv_gb300 import lespmv as L
    from sspmv_gb300 import synth
    A = synth.generate(synth.uniform(1000, 8), 1)
    M = L.csr_from_host(A)
    with pytest.raises(L.SSPMVError) as e:
        L.csr_to_sell_c_sigma(M, 100, 8)
    assert e.value.status == 1


@pytest.mark.parametrize("path", [p for p in CASES if "dups" in p.stem], ids=lambda p: p.stem)
def test_coo_to_csr_matches_reference(path):
    """Stable counting sort with duplicates kept, bit-exact vs the reference."""
    from sspmv_gb300 import lespmv as L
    z, meta, A = load(path)
    coo = L.coo_from_host(A.num_rows, A.num_cols, z["in_coo_row"], z["in_coo_col"], z["in_coo_val"])
    assert coo.s.row_sorted == 0
    out = L.coo_to_csr(coo).export()
    for k, d in meta["coo_to_csr"].items():
        assert digest(out[k]) == d, k


def test_unsorted_coo_spmv(oracle_lib):
    from sspmv_gb300 import lespmv as L
    from sspmv_gb300 import synth
    A = synth.generate(synth.powerlaw(8000, 1.8, 16, 4000, 0.1), 5)
    rows = np.repeat(np.arange(A.num_rows, dtype=np.int32), np.diff(A.row_offset))
    perm = np.random.default_rng(1).permutation(A.nnz)
    coo = L.coo_from_host(A.num_rows, A.num_cols, rows[perm], A.col_index[perm], A.values[perm])
    x = synth.vector(A.num_cols, 0)
    y0 = synth.vector(A.num_rows, 3)
    y = to_dev(y0)
    L.LeSpMV(ALPHA, coo, to_dev(x), BETA, y)
    y64, absum = oracle_lib.spmm_ref(A, x, ALPHA, BETA, y0)
    ok, mx, _ = tolerance_ok(to_host(y), y64, absum, np.diff(A.row_offset), np.float64, ALPHA, BETA, y0)
    assert ok, mx


@pytest.mark.parametrize("fmt", ["csr", "coo", "sell_c_sigma", "bsr"])
def test_deterministic_bits(fmt):
    """Same bits on every run (no atomics in the sorted-format kernels)."""
    from sspmv_gb300 import lespmv as L
    from sspmv_gb300 import synth
    p = synth.block(40000, 4, 9000) if fmt == "bsr" else synth.powerlaw(60000, 1.8, 16, 40000, 0.05)
    A = synth.generate(p, 8)
    M = L.csr_from_host(A)
    G = M if fmt == "csr" else (L.csr_to_bsr(M, 4, 4) if fmt == "bsr" else getattr(L, f"csr_to_{fmt}")(M))
    x = to_dev(synth.vector(A.num_cols, 0))
    outs = []
    for _ in range(3):
        y = to_dev(np.zeros(A.num_rows))
        L.LeSpMV(1.0, G, x, 0.0, y)
        outs.append(to_host(y))
    assert all(np.array_equal(outs[0], o) for o in outs[1:])


@pytest.mark.parametrize("dt", [np.float64, np.float32], ids=["f64", "f32"])
@pytest.mark.parametrize("fmt", ["sell_c4", "scs_c8", "scr_c16", "sell"])
def test_sliced_overflow_caps(fmt, dt, oracle_lib):
    """Thread-pass caps set through sspmv_set_kernel's param (0 = cost model):
    rows longer than the cap finish in the overflow CSR pass; results stay
    within tolerance at every cap and after the cap changes."""
    from sspmv_gb300 import lespmv as L
    from sspmv_gb300 import synth
    A = synth.generate(FAMILIES["powerlaw"](synth), 3, dt)
    M = L.csr_from_host(A)
    G = GPU_CONV[fmt](L, M)
    nnz_row = np.diff(A.row_offset)
    for cap in (1, 4, 8, 33, 0, 1 << 30, 16):
        G.set_kernel(0, cap)
        for k in (1, 3, 8):
            X = synth.vector(A.num_cols, 0, dt, k).reshape(A.num_cols, k)
            Y0 = synth.vector(A.num_rows, 9, dt, k).reshape(A.num_rows, k)
            Y = to_dev(Y0)
            L.spmm(ALPHA, G, to_dev(X), BETA, Y)
            y64, absum = oracle_lib.spmm_ref(A, X, ALPHA, BETA, Y0)
            ok, mx, _ = tolerance_ok(to_host(Y), y64, absum, nnz_row, dt, ALPHA, BETA, Y0)
            assert ok, f"{fmt}/cap={cap}/k={k}: max normalised error {mx}"


def test_dia_converter_mixed_warps(oracle_lib):
    """A banded matrix with scattered extra entries in some rows: warps whose
    rows share diagonals (grouped atomics) and warps that do not (one thread
    per row) in one conversion; arrays bit-exact against the oracle."""
    from sspmv_gb300 import lespmv as L
    from sspmv_gb300 import synth
    rng = np.random.default_rng(11)
    m = 20000
    rows, cols = [], []
    for i in range(m):
        cs = {j for j in (i - 3, i - 1, i, i + 1, i + 3) if 0 <= j < m}
        if (i // 64) % 5 == 0:  # scattered entries on 40 far diagonals, after the band
            cs |= {j for j in (i + 500 + int(rng.integers(0, 40)),) if j < m}
        if (i // 32) % 7 == 3:  # whole warps whose rows start on different diagonals
            cs |= {j for j in (i - 700 - int(rng.integers(0, 40)),) if j >= 0}
        rows += [i] * len(cs)
        cols += sorted(cs)
    rows, cols = np.array(rows), np.array(cols, np.int32)
    rp = np.zeros(m + 1, np.int32)
    np.add.at(rp, rows + 1, 1)
    rp = np.cumsum(rp).astype(np.int32)
    A = synth.HostCSR(m, m, rp, cols, rng.uniform(-1, 1, len(cols)))
    ref = oracle_lib.csr_to_dia(A)
    assert ref is not None
    out = L.csr_to_dia(L.csr_from_host(A)).export()
    for name, arr in ref.items():
        if isinstance(arr, np.ndarray):
            assert np.array_equal(out[name].view(np.uint8), arr.view(np.uint8)), name


def test_readers_and_coo_to_ell(tmp_path, oracle_lib):
    """read_<fmt>_matrix (a .mtx through CSR, ELL through COO) give the
    arrays of the converters on read_csr_matrix; coo_to_ell on an unsorted COO
    equals csr_to_ell after coo_to_csr (each row in COO order)."""
    from sspmv_gb300 import lespmv as L
    from sspmv_gb300 import synth
    A = synth.generate(synth.powerlaw(3000, 1.8, 8.0, 200, 0.05), 2)
    p = tmp_path / "a.mtx"
    L.write_mtx(str(p), A)
    csr = L.csr_from_host(L.read_csr_matrix(str(p)))
    pairs = [
        (L.read_ell_matrix(str(p)), L.csr_to_ell(csr, L.RowMajor)),
        (L.read_sell_matrix(str(p), 8, 4), L.csr_to_sell(csr, 8, 4)),
        (L.read_sell_c_sigma_matrix(str(p), 256, 8, 0), L.csr_to_sell_c_sigma(csr, 256, 8, 0)),
        (L.read_sell_c_R_matrix(str(p), 16, 0), L.csr_to_sell_c_R(csr, 16, 0)),
        (L.read_bsr_matrix(str(p), 4, 4), L.csr_to_bsr(csr, 4, 4)),
        (L.read_csr5_matrix(str(p)), L.csr_to_csr5(csr)),
    ]
    for got, ref in pairs:
        a, b = got.export(), ref.export()
        for k in b:
            if isinstance(b[k], np.ndarray):
                assert np.array_equal(a[k].view(np.uint8), b[k].view(np.uint8)), (type(got).__name__, k)
    coo = L.read_coo_matrix(str(p))
    assert coo.num_nnzs == A.nnz
    rows = np.repeat(np.arange(A.num_rows, dtype=np.int32), np.diff(A.row_offset))
    perm = np.random.default_rng(3).permutation(A.nnz)
    ucoo = L.coo_from_host(A.num_rows, A.num_cols, rows[perm], A.col_index[perm], A.values[perm])
    e1 = L.coo_to_ell(ucoo).export()
    e2 = L.csr_to_ell(L.coo_to_csr(ucoo), L.RowMajor).export()
    for k in e2:
        if isinstance(e2[k], np.ndarray):
            assert np.array_equal(e1[k].view(np.uint8), e2[k].view(np.uint8)), k


@pytest.mark.parametrize("dt", [np.float64, np.float32], ids=["f64", "f32"])
def test_reference_bytes_model(dt):
    """sspmv_reference_bytes_<fmt> equals the reference's bytes_per_spmv
    (include/spmv_benchmark.h:26-150) restated here from each format's
    exported arrays: per-chunk widths of the sliced formats, occupied rows of
    an unsorted COO, BSR block counts, the CSR5 tile count."""
    from sspmv_gb300 import lespmv as L
    from sspmv_gb300 import synth
    A = synth.generate(synth.powerlaw(5000, 1.8, 8.0, 300, 0.1), 4, dtype=dt)
    M = L.csr_from_host(A)
    sv, si = np.dtype(dt).itemsize, 4
    m, nnz = A.num_rows, A.nnz
    lens = np.diff(A.row_offset)
    assert M.reference_bytes() == 2 * si * m + si * nnz + 2 * sv * nnz + 2 * sv * m
    # COO from a permuted copy: y charged for occupied rows only
    rows = np.repeat(np.arange(m, dtype=np.int32), lens)
    perm = np.random.default_rng(1).permutation(nnz)
    coo = L.coo_from_host(m, A.num_cols, rows[perm], A.col_index[perm], A.values[perm])
    occ = int(np.count_nonzero(lens))
    assert occ < m
    assert coo.reference_bytes() == 2 * si * nnz + 2 * sv * nnz + 2 * sv * occ
    ell = L.csr_to_ell(M, L.RowMajor)
    w = ell.export()["max_row_width"]
    assert ell.reference_bytes() == si * m * w + sv * m * w + sv * nnz + 2 * sv * m
    sell = L.csr_to_sell(M, 8, 4)
    e = sell.export()
    slots = int(e["row_width"].astype(np.int64).sum()) * 8
    assert sell.reference_bytes() == si * e["chunk_num"] + 2 * si * slots + sv * nnz + 2 * sv * m
    for S, C in ((L.csr_to_sell_c_sigma(M, 64, 16, 0), 16), (L.csr_to_sell_c_R(M, 32, 0), 32)):
        e = S.export()
        slots = int(e["chunk_len"].astype(np.int64).sum()) * C
        assert S.reference_bytes() == si * e["validchunkNum"] + si * m + 2 * si * slots + sv * nnz + 2 * sv * m
    dia = L.csr_to_dia(L.csr_from_host(synth.generate(synth.banded(4000, [-2, 0, 3]), 5)))
    sv_d = 8
    assert dia.reference_bytes() == 2 * sv_d * dia.num_nnzs + 2 * sv_d * 4000
    bsr = L.csr_to_bsr(M, 4, 2)
    e = bsr.export()
    assert bsr.reference_bytes() == (2 * si * e["mb"] + si * e["nnzb"] + 2 * sv * e["nnzb"] * 8 + 2 * sv * m)
    c5 = L.csr_to_csr5(M)
    e = c5.export()
    assert c5.reference_bytes() == 2 * si * m + si * nnz + 2 * sv * nnz + 2 * sv * m + si * e["p"] + si


@pytest.mark.parametrize("dt", [np.float64, np.float32], ids=["f64", "f32"])
def test_bsr_block_stream_shapes(dt, oracle_lib):
    """BSR SpMV through the block-stream kernel (kernel_flag 2; r a power of
    two <= 32, c in {1, 2, 4, 8, 16}), the thread-per-row kernel (kernel_flag
    1, and the shapes the stream kernel does not take) and the default choice: ragged last block row and
    column, empty block rows, one long block row spanning many warps' worth
    of blocks; beta = 0 and beta != 0; both within tolerance of the FP64
    product and run twice with identical bits."""
    from sspmv_gb300 import lespmv as L
    from sspmv_gb300 import synth
    A = synth.generate(synth.powerlaw(3001, 1.6, 6.0, 2999, 0.3), 11, dt)
    M = L.csr_from_host(A)
    nnz_row = np.diff(A.row_offset)
    x = synth.vector(A.num_cols, 0, dt)
    y0 = synth.vector(A.num_rows, 9, dt)
    for r, c in ((1, 1), (2, 2), (4, 4), (8, 4), (16, 8), (32, 2), (4, 16), (3, 4), (4, 3)):
        B = L.csr_to_bsr(M, r, c)
        for flag in (0, 1, 2):
            B.set_kernel(flag, 0)
            for beta in (0.0, BETA):
                outs = []
                for _ in range(2):
                    Y = to_dev(y0)
                    L.LeSpMV(ALPHA, B, to_dev(x), beta, Y)
                    outs.append(to_host(Y))
                assert np.array_equal(outs[0].view(np.uint8), outs[1].view(np.uint8)), (r, c, flag, beta)
                y64, absum = oracle_lib.spmm_ref(A, x.reshape(-1, 1), ALPHA, beta, y0.reshape(-1, 1))
                ok, mx, _ = tolerance_ok(outs[0].reshape(-1, 1), y64, absum, nnz_row, dt, ALPHA, beta,
                                         y0.reshape(-1, 1))
                assert ok, f"bsr {r}x{c} flag={flag} beta={beta}: max normalised error {mx}"


@pytest.mark.parametrize("dt", [np.float64, np.float32], ids=["f64", "f32"])
def test_plain_sum_instantiations(dt, oracle_lib):
    """alpha = 1, beta = 0 (y = sum, the kernels' multiply-free instantiation)
    through the CSR stream / vector (one and several lanes per row) / row-block,
    COO warp, CSR5 tile, BSR (block-stream and thread-per-row) and sliced
    (S-ELL, SELL-c-sigma, SELL-c-R, with their overflow passes) kernels, on
    rows that end at every position of a lane's nonzeros (power-law rows with
    empty rows), and DIA and thread-per-row BSR on a banded matrix: within
    tolerance of the FP64 product, and y fully written (a NaN-filled y comes
    back finite)."""
    from sspmv_gb300 import lespmv as L
    from sspmv_gb300 import synth
    A = synth.generate(synth.powerlaw(20000, 1.7, 5.0, 3000, 0.2), 21, dt)
    M = L.csr_from_host(A)
    nnz_row = np.diff(A.row_offset)
    x = synth.vector(A.num_cols, 0, dt)
    y64, absum = oracle_lib.spmm_ref(A, x.reshape(-1, 1), 1.0, 0.0, None)
    cases = [("csr0", M, 0), ("csr1", M, 1), ("csr3", M, 3), ("coo", L.csr_to_coo(M), 0),
             ("csr5", L.csr_to_csr5(M), 0), ("bsr", L.csr_to_bsr(M, 4, 4), 2),
             ("sell", L.csr_to_sell(M, 4, 0), 0), ("scs", L.csr_to_sell_c_sigma(M, 256, 8, 0), 0),
             ("scr", L.csr_to_sell_c_R(M, 16, 0), 0), ("bsr1", L.csr_to_bsr(M, 4, 4), 1),
             ("csr1_one_lane", M, (1, 1))]
    # DIA needs few diagonals: a banded matrix (9 diagonals, ragged first and last rows)
    B = synth.generate(synth.banded(30001), 22, dt)
    MB = L.csr_from_host(B)
    xb = synth.vector(B.num_cols, 0, dt)
    yb64, absb = oracle_lib.spmm_ref(B, xb.reshape(-1, 1), 1.0, 0.0, None)
    runs = [(name, G, flag, A, x, y64, absum, nnz_row) for name, G, flag in cases]
    runs += [("dia", L.csr_to_dia(MB), 0, B, xb, yb64, absb, np.diff(B.row_offset)),
             ("bsr1_banded", L.csr_to_bsr(MB, 4, 4), 1, B, xb, yb64, absb, np.diff(B.row_offset))]
    for name, G, flag, H, xh, yr, ab, nr in runs:
        G.set_kernel(*(flag if isinstance(flag, tuple) else (flag, 0)))
        Y = to_dev(np.full(H.num_rows, np.nan, dt))
        L.LeSpMV(1.0, G, to_dev(xh), 0.0, Y)
        y = to_host(Y)
        assert np.isfinite(y).all(), name
        ok, mx, _ = tolerance_ok(y.reshape(-1, 1), yr, ab, nr, dt, 1.0, 0.0, None)
        assert ok, f"{name}: max normalised error {mx}"


def _banded_rect(dt, m, n, offsets, seed):
    """Banded rows with the given column offsets, num_cols n (any shape)."""
    from sspmv_gb300.synth import HostCSR
    rng = np.random.default_rng(seed)
    rows, cols = [], []
    for i in range(m):
        cs = sorted({i + o for o in offsets if 0 <= i + o < n})
        rows.append(len(cs))
        cols.extend(cs)
    rp = np.concatenate([[0], np.cumsum(rows)]).astype(np.int32)
    return HostCSR(m, n, rp, np.asarray(cols, np.int32), rng.uniform(-1, 1, int(rp[-1])).astype(dt))


@pytest.mark.parametrize("dt", [np.float64, np.float32], ids=["f64", "f32"])
@pytest.mark.parametrize("shape", [(30001, 30001, (0, 1, -1, 2, -2, 1024, -1024, 2048, -2048)),
                                   (1000, 1537, (0, 3, 700, -5, 1500)),
                                   (4099, 257, (0, -1, -4000, 7, 200)),
                                   (255, 255, tuple(range(-8, 8)))],
                         ids=["banded", "wide", "tall", "sixteen_diags"])
def test_dia_staged_kernel(shape, dt, oracle_lib):
    """kernel_flag 1 of DIA (values and x windows staged in shared memory by
    bulk copies): rows not a multiple of the tile, windows cut at both ends of
    x, non-square shapes, 16 diagonals; general alpha/beta and y = sum."""
    from sspmv_gb300 import lespmv as L
    from sspmv_gb300 import synth
    m, n, offs = shape
    A = _banded_rect(dt, m, n, offs, 5)
    M = L.csr_to_dia(L.csr_from_host(A))
    M.set_kernel(1, 0)
    x = synth.vector(n, 0, dt)
    y0 = synth.vector(m, 4, dt)
    for alpha, beta, init in ((ALPHA, BETA, y0), (1.0, 0.0, np.full(m, np.nan, dt))):
        y = to_dev(init)
        L.LeSpMV(alpha, M, to_dev(x), beta, y)
        y64, absum = oracle_lib.spmm_ref(A, x, alpha, beta, y0 if beta else None)
        ok, mx, _ = tolerance_ok(to_host(y), y64, absum, np.diff(A.row_offset), dt, alpha, beta,
                                 y0 if beta else None)
        assert ok, f"{shape[:2]} alpha {alpha}: max normalised error {mx}"
    assert L.wait_timeouts() == 0


def test_dia_staged_falls_back_past_sixteen_diagonals(oracle_lib):
    """kernel_flag 1 with 17 diagonals runs the thread-per-row kernel."""
    from sspmv_gb300 import lespmv as L
    from sspmv_gb300 import synth
    A = _banded_rect(np.float64, 5000, 5000, tuple(range(-8, 9)), 6)
    M = L.csr_to_dia(L.csr_from_host(A))
    assert M.s.complete_ndiags == 17
    M.set_kernel(1, 0)
    x = synth.vector(5000, 0)
    y = to_dev(np.zeros(5000))
    L.LeSpMV(1.0, M, to_dev(x), 0.0, y)
    y64, absum = oracle_lib.spmm_ref(A, x, 1.0, 0.0)
    ok, mx, _ = tolerance_ok(to_host(y), y64, absum, np.diff(A.row_offset), np.float64)
    assert ok, mx
