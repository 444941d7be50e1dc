"""Times the reference's own 3D velocity training step on the host CPU.

Test infrastructure, development container only: it imports the reference
checkout named by ``$NEB_REFERENCE`` (required), which the GPU
machines do not have, and runs its CuPy code on NumPy through the stand-in
module of ``tests/golden/make_golden.py`` (the pattern of the reference's
tests/test_finite_gauge.py:10-16).  The step is
experiments/metaball/_backend/flow/cases/metaball/velocity/core.py:79
``compute`` (fields of per-mode SIREN jets, Grams, causal peel, recompute and
hand-written reverse pass), driven as experiments/metaball/train.py:226-229
does for the Velocity method, with the reference's configuration
experiments/metaball/configs/metaball-velocity-k32-seed0.json (K = 32 modes,
5 x 128 SIREN per mode, 6144 points per step).  The result is the
"reference algorithm on CPU" figure quoted in the design notes; it is not a
bench line (bench.py never reads the reference).

Usage:  python oracle/reference_cpu_timing.py [points]
"""
from __future__ import annotations

import importlib.util
import json
import os
import sys
import time
from pathlib import Path
from types import SimpleNamespace

ROOT = Path(__file__).resolve().parents[1]
def reference_root() -> Path:
    """The reference checkout, named by $NEB_REFERENCE (required)."""
    root = os.environ.get("NEB_REFERENCE")
    if not root:
        raise SystemExit("set NEB_REFERENCE to the reference checkout (baiming-zhang/NEB)")
    return Path(root)


def main(points: int | None = None) -> dict:
    sys.dont_write_bytecode = True
    sys.path.insert(0, str(ROOT / "tests" / "golden"))
    import make_golden as MG
    MG.install_shim()
    import numpy as np
    vendor = reference_root() / "experiments/metaball/_backend"
    case = vendor / "flow/cases/metaball"
    sys.path[:0] = [str(vendor), str(case), str(case / "velocity")]
    spec = importlib.util.spec_from_file_location("reference_train",
                                                  reference_root() / "experiments/metaball/train.py")
    train = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(train)
    cfg_path = reference_root() / "experiments/metaball/configs/metaball-velocity-k32-seed0.json"
    config = train.runtime_configuration(json.loads(cfg_path.read_text()))
    c = SimpleNamespace(**config)
    core = MG.load(case / "velocity/core.py", "reference_velocity_core")
    # the reference's train.py sets its BLAS thread variables to 1 when it is
    # imported, after NumPy has started: the pool size actually in use is
    # read back rather than taken from the environment
    from threadpoolctl import threadpool_info
    blas_threads = max((p["num_threads"] for p in threadpool_info()
                        if p.get("user_api") == "blas"), default=None)
    K = config["modes"]
    n = points or config["points_per_step"]
    model = core.Model(c, K, config["seed"])
    geo = np.asarray(c.fixed_training_geometry, "f4")
    pts = core.fluid_points(c, geo, n, c.seed + 100000)
    t0 = time.perf_counter()
    res = core.compute(model, c, geo, pts)
    seconds = time.perf_counter() - t0
    out = {"config": cfg_path.name, "K": K, "points": int(len(pts)),
           "hidden": config["hidden"], "hidden_layers": config["hidden_layers"],
           "seconds_per_step": seconds, "steps_per_s": 1.0 / seconds,
           "phases_s": {k: round(v, 3) for k, v in res["timings"].items()},
           "host_cores": os.cpu_count(), "blas_threads": blas_threads}
    print(json.dumps(out))
    return out


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else None)
