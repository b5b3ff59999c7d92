"""The reference's random draws for the device initialiser (lb_draws.h,
compiled here as host code) against numpy's Mt19937 in the order the host
initialiser consumes it (dlbc_gb300/init.py, pinned by the init-2d
goldens): per rank of the process grid, per component, one draw per haloed
site of the rank's block (ConstRandom: per population), the physical ones
kept."""
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def expected(n, halo, nc, seed, shift, per_site, reseed, rseed, comp):
    n, halo, nc = list(n), list(halo), list(nc)
    nl = [n[i] // nc[i] for i in range(3)]
    nlh = [nl[i] + 2 * halo[i] for i in range(3)]
    out = [np.zeros(tuple(n) + (max(per_site[c], 1),), np.uint32) for c in range(2)]
    for rank in range(nc[0] * nc[1] * nc[2]):
        cc = [rank // (nc[1] * nc[2]), (rank // nc[2]) % nc[1], rank % nc[2]]
        r = rank if shift else 0
        g = np.random.RandomState((seed + r) & 0xFFFFFFFF)
        for c in range(2):
            m = per_site[c]
            if m == 0:
                continue
            gen = np.random.RandomState((rseed[c] + r) & 0xFFFFFFFF) if reseed[c] else g
            u = gen.randint(0, 2 ** 32, size=int(np.prod(nlh)) * m, dtype=np.uint32).reshape(tuple(nlh) + (m,))
            phys = tuple(slice(halo[i], halo[i] + nl[i]) for i in range(3))
            dst = tuple(slice(cc[i] * nl[i], (cc[i] + 1) * nl[i]) for i in range(3))
            out[c][dst] = u[phys]
    return out[comp].reshape(-1)


CASES = [
    # n, halo, nc, seed, shift, per_site, reseed, random seeds
    ((8, 6, 4), (2, 2, 2), (1, 1, 1), 7, True, (1, 1), (False, False), (0, 0)),
    ((8, 6, 4), (2, 2, 2), (2, 1, 2), -3, True, (1, 1), (False, False), (0, 0)),
    ((12, 8, 1), (2, 2, 0), (2, 2, 1), 0, True, (1, 1), (True, True), (42, 43)),
    ((6, 4, 4), (2, 2, 2), (2, 1, 1), 5, False, (19, 1), (False, False), (0, 0)),
    ((10, 6, 1), (2, 2, 0), (1, 2, 1), 9, True, (0, 9), (False, True), (0, 77)),
    ((7, 1, 1), (2, 0, 0), (1, 1, 1), 1, True, (3, 3), (False, False), (0, 0)),
]


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path_factory.mktemp("draws") / "draws_check")
    subprocess.run([cxx, "-std=c++17", "-O1", os.path.join(HERE, "draws_check.cpp"), "-o", exe], check=True,
                   capture_output=True, text=True)
    return exe


@pytest.mark.parametrize("case", CASES)
def test_reference_draws_follow_the_reference_order(harness, tmp_path, case):
    n, halo, nc, seed, shift, per_site, reseed, rseed = case
    for comp in range(2):
        if per_site[comp] == 0:
            continue
        path = str(tmp_path / f"d{comp}.bin")
        args = [harness, path, *map(str, n), *map(str, halo), *map(str, nc), str(seed), str(int(shift)),
                *map(str, per_site), *(str(int(r)) for r in reseed), *map(str, rseed), str(comp)]
        subprocess.run(args, check=True, timeout=60)
        got = np.fromfile(path, np.uint32)
        want = expected(n, halo, nc, seed, shift, per_site, reseed, rseed, comp)
        assert got.shape == want.shape and np.array_equal(got, want), (case, comp)


def test_reference_draws_reject_an_uneven_grid(harness, tmp_path):
    args = [harness, str(tmp_path / "x.bin"), "9", "4", "4", "2", "2", "2", "2", "1", "1", "0", "1", "1", "1",
            "0", "0", "0", "0", "0"]
    assert subprocess.run(args, timeout=60).returncode == 3


def test_make_init_describes_the_reference_draws():
    """The Python side of rng = 1 (dlbc_gb300.lbgpu.make_init): the
    reference's seed, process grid, seed shift and reseeded components."""
    lbgpu = pytest.importorskip("dlbc_gb300.lbgpu")
    from lbcases import spinodal

    p = spinodal((24, 20, 16), seed=-3)
    p.nc = [2, 0, 2]
    p.shift_seed_by_rank = False
    p.random_reseed = [False, True]
    p.random_seed = [0, 43]
    ini = lbgpu.make_init(p, seed=99, reference_rng=True)
    assert ini.rng == 1 and ini.seed == (-3) & 0xFFFFFFFFFFFFFFFF
    assert list(ini.nc) == [2, 1, 2] and ini.shift_seed_by_rank == 0
    assert list(ini.random_reseed) == [0, 1] and list(ini.random_seed) == [0, 43]
    ini = lbgpu.make_init(p, seed=99)
    assert ini.rng == 0 and ini.seed == 99 and list(ini.nc) == [0, 0, 0]


def test_reference_draws_random_shapes(harness, tmp_path):
    """Twenty seeded random shapes, grids, seeds and reseed choices (3D,
    2D and 1D), both components."""
    rng = np.random.default_rng(11)
    for i in range(20):
        d = int(rng.integers(1, 4))
        nc = [int(rng.integers(1, 4)) if k < d else 1 for k in range(3)]
        n = [nc[k] * int(rng.integers(1, 5)) if k < d else 1 for k in range(3)]
        halo = [2 if k < d else 0 for k in range(3)]
        per_site = (int(rng.choice([0, 1, 3])), int(rng.choice([1, 5])))
        reseed = (bool(rng.integers(0, 2)), bool(rng.integers(0, 2)))
        rseed = (int(rng.integers(-5, 100)), int(rng.integers(-5, 100)))
        seed, shift = int(rng.integers(-1000, 1000)), bool(rng.integers(0, 2))
        case = (tuple(n), tuple(halo), tuple(nc), seed, shift, per_site, reseed, rseed)
        for comp in range(2):
            if per_site[comp] == 0:
                continue
            path = str(tmp_path / f"r{i}_{comp}.bin")
            args = [harness, path, *map(str, n), *map(str, halo), *map(str, nc), str(seed), str(int(shift)),
                    *map(str, per_site), *(str(int(r)) for r in reseed), *map(str, rseed), str(comp)]
            subprocess.run(args, check=True, timeout=60)
            got = np.fromfile(path, np.uint32)
            want = expected(n, halo, nc, seed, shift, per_site, reseed, rseed, comp)
            assert np.array_equal(got, want), (case, comp)
