"""Generates tests/golden/parity_digests.json: digests of the REFERENCE's own results on the full
benchmark workloads, for the GPU parity tests (tests/test_gpu_golden.py).

The reference is oracle/_ref/libref.so, the reference's SuBSENSE / PAWCS sources compiled against the
project-written OpenCV stand-in (oracle/refshim/build_ref.py); it can only be built where the
reference sources are present, so its results travel as digests. Per case the file holds the
BLAKE2b-128 digest of the foreground mask of every frame and, at checkpoints, of every model map
(the layouts of oracle.h, which the GPU's inspection exports reproduce) with the frame-level scalars.

Cases (synthetic seeded scenes of include/lvbgs_synth.h, identical bytes on every machine):
  subsense_config0   320x240 BGR, all 200 frames                     state every 25 frames
  subsense_config1   1920x1080 BGR, 300 of 500 frames (both stopped   state every 25 frames
                     ellipses: shape 0 stops at frames 50-150, shape 1 at 200-300)
  subsense_changedet 640x480 BGR, lr = 1 for frames <= 100 then 0    state every 25 frames
                     (apps/changedet/src/main.cpp:390), 150 frames
  pawcs_config2      640x480 single-channel thermal-like scene, all   state every 25 frames
                     300 frames
  subsense_mix64     the 64-stream benchmark mix (stream i: preset 3 index i, scene seed 1, model
                     seed 1000 + i, as bench.py), initialize + 30 frames: every stream's mask of every
                     frame (covering the benchmark's timed ticks), every stream's state at the end

Run (a few minutes, all host cores): python tests/golden/make_parity_digests.py [--impl reference|port]
"""
import argparse
import hashlib
import json
import os
import sys
import time
from concurrent.futures import ThreadPoolExecutor

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from litiv_gb300 import SyntheticStream  # noqa: E402  (host renderer only)
from oracle import pyoracle  # noqa: E402

OUT = os.path.join(HERE, "parity_digests.json")

SUB_MAPS = ["R", "V", "T", "DLAST", "DMIN_LT", "DMIN_ST", "RAW_LT", "RAW_ST", "FIN_LT", "FIN_ST", "UNSTABLE",
            "BLINKS", "LAST_RAW_FG", "LAST_FG", "LAST_FG_DIL_INV", "LAST_RAW_BLINK", "ROI", "LAST_COLOR",
            "LAST_DESC", "SAMPLE_COLOR", "SAMPLE_DESC", "LUT"]
SUB_DS_MAPS = ["DS_LT", "DS_ST"]
SUB_SCALARS = ["frame_idx", "frames_since_last_reset", "model_reset_cooldown", "auto_model_reset_enabled",
               "learning_rate_scaling_enabled", "use_3x3_spread", "median_blur_kernel_size", "lr_lower_cap",
               "lr_upper_cap", "last_nonzero_desc_ratio", "n_relevant_px", "orig_roi_px"]
PAWCS_MAPS = pyoracle.PAWCS_MAP_NAMES
PAWCS_SCALARS = ["frame_idx", "frames_since_last_reset", "model_reset_cooldown", "lword_weight_offset",
                 "auto_model_reset_enabled", "using_moving_camera", "median_blur_kernel_size", "n_local_words",
                 "n_global_words", "last_nonflat_ratio", "n_relevant_px", "orig_roi_px", "ds_roi_px"]


def digest(a):
    return hashlib.blake2b(np.ascontiguousarray(a).view(np.uint8).tobytes(), digest_size=16).hexdigest()


def sub_maps(scalars):
    return SUB_MAPS + (SUB_DS_MAPS if scalars["learning_rate_scaling_enabled"] else [])


def state_digest(model, algo):
    sc = model.scalars()
    names = sub_maps(sc) if algo == "subsense" else PAWCS_MAPS
    keys = SUB_SCALARS if algo == "subsense" else PAWCS_SCALARS
    return {"maps": {n: digest(model.state_map(n)) for n in names},
            "scalars": {k: (float(sc[k]) if isinstance(sc[k], float) else int(sc[k])) for k in keys}}


def run_sequence(impl, algo, frames, seed, lrs=None, state_every=25):
    cls = pyoracle.OracleSuBSENSE if algo == "subsense" else pyoracle.OraclePAWCS
    m = cls(seed=seed, impl=impl)
    m.initialize(frames(0))
    out = {"masks": [], "states": {"0": state_digest(m, algo)}}
    n = frames.n
    for t in range(1, n):
        mask = m.apply(frames(t), 0.0 if lrs is None else lrs[t])
        out["masks"].append(digest(mask))
        if t % state_every == 0 or t == n - 1:
            out["states"][str(t)] = state_digest(m, algo)
    m.close()
    return out


class Frames:
    def __init__(self, config, index, seed, n, **kw):
        self.s = SyntheticStream(config, index, seed, **kw)
        self.n = n

    def __call__(self, t):
        return self.s.render(t)


def case_specs():
    lr_cd = [1.0 if t <= 100 else 0.0 for t in range(150)]
    return {
        "subsense_config0": dict(algo="subsense", config=0, index=0, scene_seed=1, seed=1, n=200),
        "subsense_config1": dict(algo="subsense", config=1, index=0, scene_seed=1, seed=1, n=301),
        "subsense_changedet": dict(algo="subsense", config=0, index=0, scene_seed=7, seed=7, n=150,
                                   scene=dict(width=640, height=480), lrs=lr_cd),
        "pawcs_config2": dict(algo="pawcs", config=2, index=0, scene_seed=1, seed=1, n=300),
    }


def run_mix64(impl, n_ticks=30, threads=None):
    def one(i):
        f = Frames(3, i, 1, n_ticks + 1)
        r = run_sequence(impl, "subsense", f, 1000 + i, state_every=10 ** 9)
        r["states"] = {str(n_ticks): r["states"][str(n_ticks)]}
        return r
    with ThreadPoolExecutor(threads or os.cpu_count()) as ex:
        streams = list(ex.map(one, range(64)))
    return {"algo": "subsense", "config": 3, "scene_seed": 1, "seed_base": 1000, "ticks": n_ticks, "streams": streams}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--impl", default="reference", choices=["reference", "port"])
    ap.add_argument("--only", default=None, help="comma-separated case names")
    args = ap.parse_args()
    if args.impl == "reference" and pyoracle.ref_lib() is None:
        raise SystemExit("the reference cannot be built here (its sources are not present)")
    doc = json.load(open(OUT)) if os.path.exists(OUT) else {}
    doc["generator"] = ("tests/golden/make_parity_digests.py --impl %s (oracle/_ref: the reference's own "
                        "sources)" % args.impl if args.impl == "reference" else "the C restatement")
    doc["digest"] = "blake2b-128 of the raw bytes"
    cases = doc.setdefault("cases", {})
    only = set(args.only.split(",")) if args.only else None
    specs = case_specs()
    with ThreadPoolExecutor(len(specs)) as ex:
        futs = {}
        for name, sp in specs.items():
            if only and name not in only:
                continue
            f = Frames(sp["config"], sp["index"], sp["scene_seed"], sp["n"], **sp.get("scene", {}))
            futs[name] = ex.submit(run_sequence, args.impl, sp["algo"], f, sp["seed"], sp.get("lrs"))
        for name, fu in futs.items():
            t0 = time.time()
            r = fu.result()
            sp = specs[name]
            cases[name] = dict({k: v for k, v in sp.items() if k != "lrs"}, **r)
            print(name, "done (%.0f s)" % (time.time() - t0), flush=True)
    if not only or "subsense_mix64" in only:
        t0 = time.time()
        cases["subsense_mix64"] = run_mix64(args.impl)
        print("subsense_mix64 done (%.0f s)" % (time.time() - t0), flush=True)
    json.dump(doc, open(OUT, "w"), indent=0, sort_keys=True)


if __name__ == "__main__":
    main()
