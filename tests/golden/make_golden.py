"""Regenerates tests/golden/scenarios.json from the reference runtime.

Runs every scenario of tests/scenarios.py through the reference SNNCuda CPU
runtime compiled from its own sources (oracle/_ref/libsnnref.so, built by
`make -C oracle ref` where the reference sources are present):

  * mode 1 (a tick loop over the reference classes that also records the fire
    raster and supports the runtime toggles) produces the fixture;
  * for every scenario the unmodified reference NetworkPropagator can run
    (default processor config, no toggles), mode 0 runs the
    NetworkPropagator itself and must produce the same counters and state
    digests, which pins mode 1 to the reference.

Usage: python tests/golden/make_golden.py
"""

from __future__ import annotations

import ctypes
import json
import pathlib
import sys
import time

ROOT = pathlib.Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

from snncuda_gb300 import _abi  # noqa: E402
from scenarios import SCENARIOS, run_scenario  # noqa: E402

REF = ROOT / "oracle" / "_ref" / "libsnnref.so"
OUT = pathlib.Path(__file__).resolve().parent / "scenarios.json"


def main() -> None:
    lib = _abi.bind(str(REF))
    set_mode = ctypes.CDLL(str(REF)).snnref_set_mode
    golden = {}
    for name, make in SCENARIOS.items():
        t0 = time.time()
        set_mode(1)
        mirror = run_scenario(name, lib)
        checked = "mirror only"
        if make().default_processor:
            set_mode(0)
            real = run_scenario(name, lib, with_raster=False, with_pending=False)
            for pm, pr in zip(mirror["probes"], real["probes"]):
                for key, value in pr.items():
                    if pm[key] != value:
                        raise SystemExit(f"{name}: mirror loop differs from NetworkPropagator on {key}")
            checked = "NetworkPropagator == mirror"
        golden[name] = mirror
        last = mirror["probes"][-1]
        print(f"{name:18s} {time.time() - t0:6.1f}s  {checked:28s} delivered={last['delivered_spikes']} "
              f"fired={last['fired_spikes']}")
    OUT.write_text(json.dumps(golden, indent=1, sort_keys=True) + "\n")
    print(f"wrote {OUT}")


if __name__ == "__main__":
    main()
