"""Parameter sets for the parity tests (the benchmark workloads at small
sizes, plus the reference's own golden cases)."""
from dlbc_gb300 import params


def spinodal(n=(32, 32, 32), eq="BDist2", perturb=0.01, seed=7, d=3):
    """Two-component spinodal decomposition: rho = 0.7 + U[-perturb, perturb]
    per component, tau = 1, g = 3.6, psi = 1 - exp(-rho), periodic."""
    dq = "d3q19" if d == 3 else "d2q9"
    lines = [
        "[lattice]", f"gn = [{', '.join(str(x) for x in n[:d])}]",
        "[lb]", "components = 2", 'fieldNames = ["red", "blue"]', "tau = [1.0, 1.0]",
        f"eqdist.eqDistForm = {eq}",
        "force.enableShanChen = true", "force.gcc = [[0.0, 3.6], [3.6, 0.0]]",
        "force.psiForm = Exponential",
        f"force.globalAcc = [{', '.join(['0.0'] * d)}]",
        "init.fluidInit = [EqDistPerturb, EqDistPerturb]",
        "init.fluidDensities = [[0.7], [0.7]]",
        f"init.fluidPerturb = [{perturb}, {perturb}]",
        "[random]", f"seed = {seed}",
    ]
    return params.LBParams.from_dict(params.parse_lines(lines), dq)


def droplet_channel(n=(32, 16, 16), radius=5.0, acc=1e-6, gwc=(0.0, 0.0), eq="BDist2", tau=(1.0, 1.0), d=3):
    """Red sphere (1.0 / 0.05) in a blue bath (0.05 / 1.0), walls on the
    planes of the last axis (z = 0 and z = nz-1; y for d = 2, a disc in a
    D2Q9 channel), body force along x."""
    walls = ["[false, false]"] * (d - 1) + ["[true, true]"]
    lines = [
        "[lattice]", f"gn = [{', '.join(str(x) for x in n[:d])}]",
        "[lb]", "components = 2", 'fieldNames = ["red", "blue"]', f"tau = [{tau[0]}, {tau[1]}]",
        f"eqdist.eqDistForm = {eq}",
        "force.enableShanChen = true", "force.gcc = [[0.0, 3.6], [3.6, 0.0]]",
        f"force.gwc = [{gwc[0]}, {gwc[1]}]",
        "force.psiForm = Exponential", f"force.globalAcc = [{', '.join([str(acc)] + ['0.0'] * (d - 1))}]",
        "init.fluidInit = [EqDistSphere, EqDistSphere]",
        "init.fluidDensities = [[1.0, 0.05], [0.05, 1.0]]",
        f"init.initRadius = {radius}", "init.interfaceThickness = 0.0",
        "mask.maskInit = Walls",
        f"mask.dimensionHasWall = [{', '.join(walls)}]",
        "mask.wallThickness = 1",
    ]
    return params.LBParams.from_dict(params.parse_lines(lines), "d3q19" if d == 3 else "d2q9")


# D3Q19 velocities in the reference's order (src/dlbc/lb/connectivity.d:401-418)
D3Q19_VELOCITIES = [(0, 0, 0), (1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1),
                    (1, 1, 0), (-1, 1, 0), (0, 1, 1), (0, -1, 1), (1, 0, 1), (1, 0, -1), (1, -1, 0),
                    (-1, -1, 0), (0, 1, -1), (0, -1, -1), (-1, 0, 1), (-1, 0, -1)]
