"""Host check of the FP32 face clipper: the shared-pool clipper against the local-memory
clipper on seeded random faces (tests/clip_host_check.cu, compiled for the host from the
library's csrc/fia_clip32.cuh).  No GPU: the kernels' clipping code itself, run on the CPU.
The GPU counterpart compares whole steps with the shared path on and off
(test_gpu_fp32.py::test_fp32_clip_shared_pool_matches_local_pool)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    return None


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    exe = nvcc()
    if exe is None:
        pytest.skip("nvcc not found")
    out = str(tmp_path_factory.mktemp("clip") / "clip_host_check")
    # no contraction on the host: both clippers then round every operation alike
    subprocess.check_call([exe, "-std=c++17", "-O2", "-x", "cu", "-Xcompiler", "-ffp-contract=off",
                           "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "clip_host_check.cu"),
                           "-o", out])
    return out


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_shared_pool_clipper_matches_local_clipper(checker, seed):
    r = subprocess.run([checker, "400000", str(seed)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    f = dict(zip(r.stdout.split()[0::2], (int(x) for x in r.stdout.split()[1::2])))
    assert f["mismatches"] == 0
    # the shared pool takes most faces, including non-convex ones clipped from both sides
    assert f["accepted"] > 0.7 * f["faces"]
    assert f["multi"] > 0
    assert f["listed"] > 0


def test_fp32_clipper_pieces_match_the_oracle(checker, tmp_path):
    """The FP32 clipper's pieces (local-memory store; the shared store is bitwise equal to it,
    above) against the FP64 oracle's split_face (the reference's facecutter restated) on seeded
    faces of all three families, rigid and mildly deformed, up to CFL 2.  The same pieces in
    reverse order: the kernels' explicit stack pops the last part of a cut first, the
    reference's recursion finishes the first part first; each face's piece fluxes are summed
    with compensation, so the order changes a flux by rounding only.  Y-normals to FP32
    rounding; centroids to FP32 rounding where they carry weight (a sliver piece near a corner
    has an ill-conditioned centroid and a y-normal near zero, so its error is weighted by its
    y-normal, as in the flux it contributes to)."""
    np = pytest.importorskip("numpy")
    from oracle import Oracle
    O = Oracle()
    rng = np.random.default_rng(11)
    corners = {0: [(0, 0, 0), (0, 1, 0), (0, 1, 1), (0, 0, 1)], 1: [(0, 0, 0), (0, 0, 1), (1, 0, 1), (1, 0, 0)],
               2: [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0)]}
    faces, recs = [], []
    for t in range(3000):
        fam = t % 3
        T = rng.uniform(-2.0, 2.0, size=3)
        v = np.array(corners[fam], float) + T + rng.uniform(-0.1, 0.1, size=(4, 3))
        v = v.astype(np.float32).astype(np.float64)       # the same corners in both
        off = (0.5, 0.5) if rng.integers(2) else (0.0, 0.0)
        faces.append((v, off))
        recs.append(np.concatenate([v.ravel(), off, [1.0]]).astype(np.float32))
    fin, fout = str(tmp_path / "faces.bin"), str(tmp_path / "pieces.bin")
    np.concatenate(recs).tofile(fin)
    subprocess.check_call([checker, "dump", fin, fout])
    raw = open(fout, "rb").read()
    pos, compared, pieces = 0, 0, 0
    for v, off in faces:
        n, multi = np.frombuffer(raw, np.int32, 2, pos)
        pos += 16
        p32 = np.frombuffer(raw, np.float32, 4 * n, pos).reshape(n, 4).astype(np.float64)
        pos += 16 * n
        if multi:
            continue       # clipped from both sides: the oracle's split_face returns one side
        p64, st = O.split_face(v, 1.0, off)
        assert st == 0
        p64 = p64[p64[:, 4] != 0.0][::-1]        # no piece with a zero y-normal; reverse order
        assert len(p64) == n
        ny64 = p64[:, 4]
        np.testing.assert_allclose(p32[:, 3], ny64, rtol=0, atol=2e-5)
        err = np.abs(p32[:, :3] - p64[:, :3]).max(axis=1)
        assert np.all(err * np.abs(ny64) < 1e-6)
        assert np.all(err[np.abs(ny64) > 1e-2] < 2e-5)
        compared += 1
        pieces += n
    assert pos == len(raw)
    assert compared > 2900 and pieces > 2 * compared


@pytest.mark.parametrize("cfl", [2.0, 4.0])
def test_fp32_triangulated_pieces_match_the_oracle(checker, tmp_path, cfl):
    """With minimal_area 0.05 the pieces are triangulated by longest-edge bisection
    (facecutter.h:255-324).  The fan triangles of a square have equally long edges; both the
    FP32 clipper and the oracle take lengths within a relative 4e-6 as equal and bisect the
    first, so their triangles agree, and with them each face's y-normal sum and volume point
    (sum of y n_y), which depend on the partition of a warped face.  Deformed faces up to the
    given CFL, both colour offsets."""
    np = pytest.importorskip("numpy")
    from oracle import Oracle
    O = Oracle()
    rng = np.random.default_rng(5)
    corners = {0: [(0, 0, 0), (0, 1, 0), (0, 1, 1), (0, 0, 1)], 1: [(0, 0, 0), (0, 0, 1), (1, 0, 1), (1, 0, 0)],
               2: [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0)]}
    faces, recs = [], []
    for t in range(1500):
        fam = t % 3
        T = rng.uniform(-cfl, cfl, size=3)
        v = (np.array(corners[fam], float) + T + rng.uniform(-0.3, 0.3, size=(4, 3))).astype(np.float32)
        v = v.astype(np.float64)
        off = (0.5, 0.5) if rng.integers(2) else (0.0, 0.0)
        faces.append((v, off))
        recs.append(np.concatenate([v.ravel(), off, [0.05]]).astype(np.float32))
    fin, fout = str(tmp_path / "faces.bin"), str(tmp_path / "pieces.bin")
    np.concatenate(recs).tofile(fin)
    subprocess.check_call([checker, "dump", fin, fout])
    raw = open(fout, "rb").read()
    pos, compared, triangulated = 0, 0, 0
    for v, off in faces:
        n, multi = np.frombuffer(raw, np.int32, 2, pos)
        pos += 16
        p32 = np.frombuffer(raw, np.float32, 4 * n, pos).reshape(n, 4).astype(np.float64)
        pos += 16 * n
        if multi:
            continue
        p64, st = O.split_face(v, 1.0, off, 0.05, 1024)
        assert st == 0
        p64 = p64[p64[:, 4] != 0.0]
        assert abs(p32[:, 3].sum() - p64[:, 4].sum()) < 2e-5
        assert abs((p32[:, 1] * p32[:, 3]).sum() - (p64[:, 1] * p64[:, 4]).sum()) < 2e-5
        compared += 1
        triangulated += len(p64) > 8
    assert pos == len(raw)
    assert compared > 1400 and triangulated > 1000


def test_status_words_of_the_clipper(checker):
    """The status bits that replace the reference's exit(0) in the face clipper
    (facecutter.h:191-204) and its fixed-size arrays (facecutter.h:29), on the host:
    a NaN or infinite vertex coordinate (a non-finite velocity upstream) gives
    FIA_STATUS_NONFINITE and no piece, without clipping (the clip loops are bounded by the
    range of finite colours, which such a vertex would break); a face spanning more pieces
    than a face's store holds gives FIA_STATUS_CLIP_OVERFLOW and stops at the full store,
    also for absurd finite colours (10^7 cells).  The shared-pool clipper hands every such
    face to the local-memory clipper, which sets the bits.  FIA_STATUS_CLIP_ODD_CUT cannot
    arise from these clippers' sign test (every vertex lies on one side of an iso-line, so a
    closed polygon crosses it an even number of times); its check is defensive.  The run
    ending within the timeout is part of the test."""
    r = subprocess.run([checker, "status"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    rows = {f[0]: tuple(int(x) for x in f[1:]) for f in (line.split() for line in r.stdout.splitlines())}
    NONFINITE, OVERFLOW = 4, 1
    assert rows["normal"] == (0, 4, 1)
    for name in ("nan_x", "nan_y", "inf_z", "neg_inf_x", "all_nan"):
        st, pieces, fast_ok = rows[name]
        assert st == NONFINITE and pieces == 0 and fast_ok == 0, (name, rows[name])
    for name in ("stretched", "huge"):
        st, pieces, fast_ok = rows[name]
        assert st & OVERFLOW and pieces == 128 and fast_ok == 0, (name, rows[name])
