"""Seeded inputs of the golden cases.  make_golden.py runs the reference's
own code on them; test_golden.py runs the oracle on the same inputs."""
from __future__ import annotations

import hashlib
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "casm-hella_gb300"))
import synth  # noqa: E402

NCHAN = 256  # the reference's NCHAN for these fixtures

FLAG_CASES = [
    dict(name="noise_rfi_slope_dead", seed=4, w=2048, rfi=(3, 50), slope=0.4, dead=(77,), scrunch=()),
    dict(name="burst_spikes", seed=8, w=4096, rfi=(200,), slope=-0.3, dead=(), scrunch=(), burst=True),
    dict(name="short_gulp", seed=15, w=512, rfi=(), slope=0.0, dead=(0, 255), scrunch=()),
    dict(name="scrunch_two", seed=16, w=2048, rfi=(9, 140), slope=0.2, dead=(), flag1=10, flag2=20,
         scrunch=((4, 4, 5.0, 1), (16, 2, 6.0, 1))),
    dict(name="scrunch_odd_box", seed=23, w=1024, rfi=(30,), slope=0.0, dead=(), flag1=-1, flag2=-1,
         scrunch=((3, 5, 4.0, 1),)),
]


def flag_input(c: dict) -> np.ndarray:
    sky = synth.Sky(NCHAN, 1.048576e-3, 468.75, -93.75 / NCHAN, seed=c["seed"], rfi_chans=c["rfi"], slope=c["slope"])
    if c.get("burst"):
        sky.bursts = [synth.Burst(c["w"] // 3, 60.0, 3.0, 40.0, 0.0)]
        sky.spikes = [synth.Spike(c["w"] // 2, 4, 70.0)]
    x = sky.gulp(0, c["w"])
    for d in c["dead"]:
        x[:, d] = 0
    return x


STAT_CASES = [dict(seed=1, h=40, w=700, stride=704), dict(seed=2, h=17, w=1024, stride=1024),
              dict(seed=3, h=300, w=256, stride=300)]


def stat_input_f32(c: dict) -> np.ndarray:
    rng = np.random.default_rng(c["seed"])
    return (rng.standard_normal((c["h"], c["stride"])) * 3 + 5).astype(np.float32)


def stat_input_f16(c: dict) -> np.ndarray:
    rng = np.random.default_rng(100 + c["seed"])
    return rng.uniform(0, 4, (c["h"], c["stride"])).astype(np.float16).view(np.uint16)


MEDIAN_CASES = [dict(seed=5, size=257, window=1), dict(seed=6, size=257, window=3),
                dict(seed=7, size=300, window=7), dict(seed=8, size=64, window=5)]


def median_input(c: dict) -> np.ndarray:
    return np.random.default_rng(c["seed"]).standard_normal(c["size"]).astype(np.float32)


SMOOTH_CASES = [dict(seed=31, ndms=24, ntime_out=2048, wmin=1, wmax=64, snr=3.0),
                dict(seed=32, ndms=12, ntime_out=1024, wmin=2, wmax=32, snr=2.5)]


def smooth_input(c: dict) -> np.ndarray:
    """A dedispersed plane of integer sums with a bright ridge."""
    rng = np.random.default_rng(c["seed"])
    ntd = c["ntime_out"] + c["wmax"]
    dd = np.rint(rng.normal(128 * 256, 320, (c["ndms"], ntd))).astype(np.float32)
    t0 = ntd // 3
    for d in range(c["ndms"]):
        w = max(1, 6 - abs(d - c["ndms"] // 2))
        dd[d, t0:t0 + w] += 2400.0
    return dd


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def bits(a) -> list[int]:
    return np.ascontiguousarray(np.asarray(a, np.float32)).view(np.uint32).ravel().tolist()
