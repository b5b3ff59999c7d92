"""Host-side initialisers (dlbc_gb300.init) against the oracle's restatement
and the reference's init goldens."""
import os

import numpy as np
import pytest

from dlbc_gb300 import init, params
from golden_util import GOLDEN, load_case, sha
from oracle import oracle as orc

CASES = ["merging-droplets-3d", "bdist2-sc-3d", "laplace-droplet-3d", "merging-droplets-2d",
         "bdist2-sc-2d", "poiseuille-2d", "laplace-quasi-1d-d2q9"]


@pytest.mark.parametrize("name", CASES)
def test_host_init_equals_oracle_init(name):
    z, p = load_case(name)
    fl, m = init.init_fields(p)
    o = orc.Oracle(p)
    for c in range(p.components):
        assert sha(fl[c]) == sha(o.fluid_haloed(c))
    assert np.array_equal(m, o.mask_haloed())


def test_host_init_matches_init_goldens():
    z = np.load(os.path.join(GOLDEN, "init-2d.npz"))
    keys = [str(k) for k in z["keys"]]
    for case in z["cases"]:
        case = str(case)
        p = params.LBParams.from_dict(params.parse_lines(str(z[case + "/input"]).splitlines()), "d2q9")
        fl, m = init.init_fields(p)
        phys = (slice(2, -2), slice(2, -2))
        for key in keys:
            if not key.startswith(case + "/"):
                continue
            kind = key.split("/")[1]
            if kind.startswith("population-"):
                c = p.field_names.index(kind.split("-", 1)[1])
                assert sha(fl[c][phys]) == str(z[key + "/sha256"]), key
            elif kind == "mask":
                assert sha(m[phys]) == str(z[key + "/sha256"]), key


def test_periodic_halo_fill():
    a = np.arange(6 * 5 * 4, dtype=np.float64).reshape(6, 5, 4, 1)
    h = init.periodic_fill(np.pad(a, [(2, 2), (2, 2), (2, 2), (0, 0)]), 3)
    assert h.shape == (10, 9, 8, 1)
    assert h[0, 2, 2, 0] == a[4, 0, 0, 0] and h[9, 8, 7, 0] == a[1, 1, 1, 0]


def test_mask_from_file_matches_goldens(tmp_path, monkeypatch):
    """maskInit = File (src/dlbc/lb/mask.d:153-155) on the reference's
    mask-init-file-2d input (2x2 process grid): the t = 0 dumps equal the
    reference's goldens bit for bit."""
    import os
    from dlbc_gb300 import h5
    from golden_util import GOLDEN, sha
    from oracle import oracle as orc
    z = np.load(os.path.join(GOLDEN, "init-2d.npz"))
    case = "mask-init-file-2d"
    text = str(z[f"file/{case}/input"])
    (tmp_path / "reference-data").mkdir()
    h5.write_field(str(tmp_path / "reference-data" / f"mask-{case}-t00000000.h5"), z[f"file/{case}/mask"])
    monkeypatch.chdir(tmp_path)
    p = params.LBParams.from_dict(params.parse_lines(text.splitlines()), "d2q9")
    fl, m = init.init_fields(p)
    phys = (slice(2, -2), slice(2, -2))
    assert sha(m[phys]) == str(z[f"file/{case}/mask/sha256"])
    for c, nm in enumerate(p.field_names):
        assert sha(fl[c][phys]) == str(z[f"file/{case}/population-{nm}/sha256"])
    # the colour dump: rho_red - rho_blue, 0 on solid sites
    o = orc.Oracle(p, init=False)
    for c in range(2):
        o.set_fluid_haloed(c, fl[c])
    o.set_mask_haloed(m)
    assert sha(o.colour(0, 1)) == str(z[f"file/{case}/colour/sha256"])


@pytest.mark.parametrize("nc", [[1, 1], [2, 2]])
def test_fluid_from_file(tmp_path, monkeypatch, nc):
    """fluidInit = File (src/dlbc/lb/init.d:272-275): the populations of
    every process's block come from the file; solid sites are then set to
    (1, 0, ...) as after any initialiser."""
    from dlbc_gb300 import h5
    rng = np.random.default_rng(1)
    pops = [rng.random((16, 12, 9)) for _ in range(2)]
    for i, a in enumerate(pops):
        h5.write_field(str(tmp_path / f"pop{i}.h5"), a)
    monkeypatch.chdir(tmp_path)
    lines = ["[lattice]", "gn = [16, 12]", "[parallel]", f"nc = [{nc[0]}, {nc[1]}]", "[lb]", "components = 2",
             'fieldNames = ["red", "blue"]', "init.fluidInit = [File, File]",
             'init.fluidFiles = ["pop0.h5", "pop1.h5"]', "mask.maskInit = Walls",
             "mask.dimensionHasWall = [[false, false], [true, false]]"]
    p = params.LBParams.from_dict(params.parse_lines(lines), "d2q9")
    fl, m = init.init_fields(p)
    phys = (slice(2, -2), slice(2, -2))
    for c in range(2):
        got = fl[c][phys]
        solid = m[phys] == 1
        assert np.array_equal(got[~solid], pops[c][~solid])
        assert np.all(got[solid][:, 0] == 1.0) and np.all(got[solid][:, 1:] == 0.0)
    # a file of another lattice size is rejected
    h5.write_field(str(tmp_path / "small.h5"), np.zeros((8, 12, 9)))
    bad = params.LBParams.from_dict(params.parse_lines(lines[:-4] + ["init.fluidInit = [File, File]",
                                                                     'init.fluidFiles = ["pop0.h5", "small.h5"]']),
                                    "d2q9")
    with pytest.raises(ValueError):
        init.init_fields(bad)
