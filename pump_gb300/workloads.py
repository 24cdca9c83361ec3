"""Synthetic planning problems in the reference's input-file format.

The reference reads one CSV file per query (README.md:10-11, parsed at
mainPUMP.cu:152-230): init state, goal state, lower and upper state bounds
(6 values each), the noise multiplier, the obstacle count, then 12 values per
axis-aligned box (lower corner, upper corner, 6D).  The generators below
produce the workloads the benchmarks are quoted on, seeded and reproducible:

- ``random_boxes`` -- N samples in pos [0,1]^3 x vel [-1,1]^3, init
  (0.1,0.1,0.1,0,0,0), goal (0.9,0.9,0.9,0,0,0), boxes with position centres
  U[0.2,0.8] and sides U[lo,hi] spanning the whole velocity range (+-3.1, as
  the reference's example files).
- ``indoor`` -- the same bounds with 30 walls 0.02 thick and U[0.3,1] long on
  the lines of a 4 x 4 room grid (full height), plus 10 boxes with sides
  U[0.05,0.15].
- ``large_boxes`` -- 200 boxes with centres U[0,1] and sides U[0.02,0.1].

Boxes that contain the init or goal position are redrawn.  Seeds follow
1000 * config + query.
"""
from __future__ import annotations

import numpy as np

INIT = (0.1, 0.1, 0.1, 0.0, 0.0, 0.0)
GOAL = (0.9, 0.9, 0.9, 0.0, 0.0, 0.0)
LO = (0.0, 0.0, 0.0, -1.0, -1.0, -1.0)
HI = (1.0, 1.0, 1.0, 1.0, 1.0, 1.0)
VEL = 3.1


def _contains(box, p):
    return all(box[d] < p[d] < box[6 + d] for d in range(3))


def _box(lo3, hi3):
    return [lo3[0], lo3[1], lo3[2], -VEL, -VEL, -VEL, hi3[0], hi3[1], hi3[2], VEL, VEL, VEL]


def random_boxes(n, seed, side=(0.05, 0.2), centre=(0.2, 0.8)):
    rng = np.random.Generator(np.random.MT19937(seed))
    out = []
    while len(out) < n:
        c = rng.uniform(centre[0], centre[1], 3)
        s = rng.uniform(side[0], side[1], 3)
        b = _box(c - s / 2, c + s / 2)
        if _contains(b, INIT) or _contains(b, GOAL):
            continue
        out.append(b)
    return np.asarray(out, np.float32).reshape(-1, 12)


def indoor(seed, walls=30, boxes=10):
    rng = np.random.Generator(np.random.MT19937(seed))
    out = []
    while len(out) < walls:
        k = int(rng.integers(1, 4)) / 4.0
        length = rng.uniform(0.3, 1.0)
        start = rng.uniform(0.0, 1.0 - length)
        if rng.integers(0, 2) == 0:  # wall in a plane x = k
            b = _box((k - 0.01, start, 0.0), (k + 0.01, start + length, 1.0))
        else:  # wall in a plane y = k
            b = _box((start, k - 0.01, 0.0), (start + length, k + 0.01, 1.0))
        if _contains(b, INIT) or _contains(b, GOAL):
            continue
        out.append(b)
    rest = random_boxes(boxes, seed + 7919, side=(0.05, 0.15))
    return np.concatenate([np.asarray(out, np.float32).reshape(-1, 12), rest], 0)


def write_input(path, obstacles, offset_mult, init=INIT, goal=GOAL, lo=LO, hi=HI):
    """Writes a problem in the reference's input format."""
    def row(v):
        return ",".join("%.9g" % float(x) for x in v) + ",\n"
    obstacles = np.asarray(obstacles, np.float32).reshape(-1, 12)
    with open(path, "w") as f:
        f.write(row(init) + row(goal) + row(lo) + row(hi))
        f.write("%.9g,\n%d,\n" % (offset_mult, obstacles.shape[0]))
        for k, b in enumerate(obstacles):
            line = ", ".join("%.9g" % float(x) for x in b)
            f.write(line + (",\n" if k + 1 < obstacles.shape[0] else "\n"))


def free_point(rng, obstacles):
    """A position uniform in [0,1]^3 outside every box, zero velocity."""
    while True:
        p = rng.uniform(0.0, 1.0, 3)
        if not any(_contains(b, p) for b in obstacles):
            return (float(p[0]), float(p[1]), float(p[2]), 0.0, 0.0, 0.0)


# Waypoints per edge of the batched workload: by edge length, at most
# BATCH_DISC_LEN apart in position, between 4 and 32 per edge (num_disc 3..31)
BATCH_DISC_LEN, BATCH_DISC_MIN, BATCH_DISC_MAX = 0.025, 3, 31


def batch_queries(n=256, seed=2000, n_range=(500, 8000), obs_range=(5, 100)):
    """The batched workload: per query N log-uniform in n_range, a box count
    uniform in obs_range (boxes as random_boxes), init and goal uniform in free
    space, CP target from {0.001, 0.01, 0.05}, eta from {1, 2, 4}; waypoints
    per edge by edge length (disc_len, disc_min, num_disc: 4 to 32)."""
    rng = np.random.Generator(np.random.MT19937(seed))
    out = []
    for q in range(n):
        N = int(round(np.exp(rng.uniform(np.log(n_range[0]), np.log(n_range[1])))))
        nobs = int(rng.integers(obs_range[0], obs_range[1] + 1))
        obs = random_boxes(nobs, seed * 1000 + q)
        init = free_point(rng, obs)
        goal = free_point(rng, obs)
        out.append(dict(N=N, obstacles=obs, init=init, goal=goal,
                        cp=float(rng.choice([0.001, 0.01, 0.05])),
                        eta=float(rng.choice([1.0, 2.0, 4.0])), offset_mult=np.float32(1e-3),
                        disc_len=BATCH_DISC_LEN, disc_min=BATCH_DISC_MIN, num_disc=BATCH_DISC_MAX))
    return out


def perturbed_paths(n_paths, seed, obstacles, n_range=(8, 40), spread=0.05, speed=0.3):
    """Paths for the refinement objective: node count uniform in n_range,
    free init and goal at rest, intermediate positions on the straight line
    plus a sin-shaped Gaussian detour of scale `spread`, velocities
    N(0, speed^2).  Returns (nodes (rows, 6) float32, offsets, counts)."""
    rng = np.random.Generator(np.random.MT19937(seed))
    rows, offs, cnts = [], [], []
    total = 0
    for _ in range(n_paths):
        n = int(rng.integers(n_range[0], n_range[1] + 1))
        a, b = free_point(rng, obstacles), free_point(rng, obstacles)
        s = np.linspace(0.0, 1.0, n)[:, None]
        X = np.zeros((n, 6))
        X[:, :3] = a[:3] * (1 - s) + b[:3] * s + rng.normal(0, spread, (n, 3)) * np.sin(np.pi * s)
        X[:, 3:] = rng.normal(0, speed, (n, 3))
        X[0, :3], X[-1, :3] = a[:3], b[:3]
        X[0, 3:] = X[-1, 3:] = 0
        rows.append(X.astype(np.float32))
        offs.append(total)
        cnts.append(n)
        total += n
    return np.concatenate(rows), np.asarray(offs, np.int32), np.asarray(cnts, np.int32)


def large_boxes(seed, n=200):
    """The large configuration's map: n boxes with position centres U[0, 1]
    and sides U[0.02, 0.1] (spanning the velocity range)."""
    return random_boxes(n, seed, side=(0.02, 0.1), centre=(0.0, 1.0))


CONFIGS = {
    # the benchmark configurations (N, obstacles, noise, cp, eta, particles, waypoints)
    "cfg0": dict(N=1000, num_disc=9, num_hsmc=128, offset_mult=1e-3, cp=0.01, eta=2.0,
                 obstacles=lambda q=0: random_boxes(10, 1000 * 0 + q)),
    "cfg1": dict(N=4000, num_disc=8, num_hsmc=1024, offset_mult=2e-3, cp=0.01, eta=2.0,
                 obstacles=lambda q=0: indoor(1000 * 1 + q)),
    # the large configuration: 4096 particles for HSMC and for the Monte Carlo CP.
    # Its fourth wavefront holds 14.1 M new paths, past the reference's path
    # store of 2 N sqrt(N) = 11.4 M (where the reference ends the search,
    # PUMP.cu:62-76), so the store is 2^24 paths.
    "cfg4": dict(N=32000, num_disc=15, num_hsmc=4096, num_mc=4096, offset_mult=5e-3, cp=0.005,
                 eta=2.0, max_paths=1 << 24, obstacles=lambda q=0: large_boxes(1000 * 4 + q)),
}
