"""Generate tests/golden/golden.npz from the CPU oracle.

The reference ships no golden vectors for this path (parity unpinned), so
these fixtures freeze the oracle's restatement: point physics on seeded
states and a short run on a small grid. Regenerate only on a deliberate
change of the restated algorithm:

    python tests/golden/make_golden.py
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "app-kilonova_gb300"))
sys.path.insert(0, str(ROOT / "oracle"))

import knc_oracle as ko  # noqa: E402
from knc import config  # noqa: E402


def small_grid():
    hydro = config.RelativisticHydro(4.0 / 3.0, 1.5, 0.4, "RK2", "HLLE")
    mesh = config.Mesh(reference_radius=1.0, inner_radius=1.0, outer_radius=2.0, inner_excision_speed=0.0,
                       outer_excision_speed=0.0, num_polar_zones=16, block_size=8, num_radial_zones=16)
    model = config.WindModel(seed=5)
    return hydro, mesh, model


def main():
    ko.build()
    rng = np.random.default_rng(1234)
    n = 64
    W = np.exp(rng.uniform(0, np.log(200), n))
    T = np.exp(rng.uniform(np.log(1e-5), np.log(10), n))
    rho = np.exp(rng.uniform(np.log(1e-2), np.log(1e2), n))
    ang = rng.uniform(0, 2 * np.pi, n)
    um = np.sqrt(W * W - 1)
    prims = np.stack([rho, um * np.cos(ang), um * np.sin(ang), T * rho], axis=1)
    out = {"prims": prims}
    for name, hp in [("hlle", config.RelativisticHydro(4 / 3, 1.5, 0.4, "RK2", "HLLE").to_c()),
                     ("hllc", config.RelativisticHydro(4 / 3, 1.5, 0.4, "RK2", "HLLC").to_c())]:
        cons = np.array([ko.prim_to_cons(hp, p) for p in prims])
        rec = np.array([ko.cons_to_prim(hp, u)[1] for u in cons])
        its = np.array([ko.cons_to_prim(hp, u)[2] for u in cons])
        fl = np.array([[ko.riemann(hp, prims[k], prims[(k + 1) % n], 0.2, 0.7, ax) for ax in (0, 1)]
                       for k in range(n)])
        src = np.array([ko.sources(hp, p, 1.7, 0.3) for p in prims])
        out[f"{name}_cons"], out[f"{name}_rec"], out[f"{name}_iters"] = cons, rec, its
        out[f"{name}_flux"], out[f"{name}_src"] = fl, src
    hydro, mesh, model = small_grid()
    o = ko.Oracle(hydro, mesh, threads=2)
    o.set_model(model)
    o.init_from_model(0.0)
    idx = o.block_indexes()
    out["grid_blocks"] = np.array(idx)
    out["grid_init"] = np.stack([o.get_block(i)[0] for i in idx])
    o.advance(5)
    out["grid_cons"] = np.stack([o.get_block(i)[0] for i in idx])
    out["grid_scalar"] = np.stack([o.get_block(i)[1] for i in idx])
    t, (num, den) = o.time()
    out["grid_time"] = np.array([t, num, den])
    np.savez_compressed(Path(__file__).with_name("golden.npz"), **out)
    print("wrote", Path(__file__).with_name("golden.npz"))


if __name__ == "__main__":
    main()
