"""Generate the golden fixtures in tests/golden/ from the reference nsPipe-CUDA build.

Run on a GPU host (the reference is CUDA-only):

    python tests/golden/make_golden.py OUTDIR [cfg ...]

For each configuration it writes seeded restart files (u?_s.bin), builds the
reference with that configuration's #defines (oracle/ref/build_ref.py), runs it
in 'trace' mode (one integrate() call per step, corrector iteration counts
recorded) and reduces the snapshots it writes to fixtures:

  * small configurations (s1, s2): full spectral fields at selected steps;
  * c0 (NR=48, 32x64 modes), c1 and c1h (NR=96, 128x256 modes; c1h with half
    c1's time step, 500 steps), c4b (NR=64, 48x128) and c4c (NR=96, 96x192): the low-mode block
    |m| <= 4, l <= 5 at every radius, the mean profile u_z(0,0,r), the per-
    component L2 norms and 8 seeded random projections of every component
    (a checksum of the whole field).

'io_s2' runs s2 from its seeded field for 100 steps in the 'io' mode (output
schedule build_ref.IO_SCHEDULE: rows every 0.015 / 0.05 / 0.035 time units, 4
rows per write) and keeps the four files integrate() writes, io_friction.txt,
io_qcross.txt, io_ucross.txt and io_meanpr.txt, as written (tests/golden/io_s2/).

'remesh' runs the reference Re_Mesh tool (tools/Re_Mesh/src, built by
build_ref.build_remesh with a driver main of its own) on seeded fields for the
cases in REMESH_CASES and keeps input seeds and outputs (tests/golden/remesh.npz).
The inputs are uniform in [-1, 1) from SplitMix64 (remesh_input), so they are
regenerated bit for bit from the seed.

The projections use real weights w ~ N(0,1) from SplitMix64(seed ^ 0x5bd1e995):
p = sum_h w_h u_h over the flattened field.
"""
import json
import os
import shutil
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "nspipe-gpu_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle", "ref"))
from nspipe_gb300.initfield import PI2, SplitMix64, read_state, seeded_field, write_state  # noqa: E402
import build_ref  # noqa: E402

# name -> amplitude, seed, total steps, snapshot steps, full-field fixture?
RUNS = {
    "s1": (0.05, 11, 20, [1, 5, 20], True),
    "s2": (0.1, 12, 20, [1, 10, 20], True),
    "c0": (1e-3, 2000, 100, [1, 10, 50, 100], False),
    "c1": (0.1, 5300, 100, [1, 10, 50, 100], False),
    "c1h": (0.1, 5300, 500, [1, 10, 50, 100, 200, 300, 400, 500], False),
    # one member of each larger group of the uneven mixed batch (NR=64 x 48 x 128 modes,
    # NR=96 x 96 x 192 modes; dt = 0.003 R/U_b, amplitude 0.05)
    "c4b": (0.05, 4100, 100, [1, 10, 50, 100], False),
    "c4c": (0.05, 4200, 100, [1, 10, 50, 100], False),
}
N_PROJ = 8


def projection_weights(size, seed):
    rng = np.random.default_rng(seed ^ 0x5BD1E995)
    return rng.standard_normal((N_PROJ, size))


def reduce_field(u, seed):
    NR, NT, NZ = u[0].shape
    m_slots = [0, 1, 2, 3, 4, NT - 4, NT - 3, NT - 2, NT - 1]
    w = projection_weights(u[0].size, seed)
    out = {
        "low": np.stack([a[:, m_slots, :6] for a in u]),
        "mean": u[2][:, 0, 0].copy(),
        "norm": np.array([np.linalg.norm(a) for a in u]),
        "proj": np.stack([w @ a.reshape(-1) for a in u]),
    }
    return out


# name -> old (NR, NT, NZ), new (Nrd, Ntd, Nzd), iw, seed: refinement in every
# direction, coarsening in every direction (theta and z truncation), a radial-only
# refinement with a 4-point stencil.
REMESH_CASES = {
    "up": ((24, 8, 9), (32, 12, 13), 3, 101),
    "down": ((32, 16, 17), (24, 8, 9), 3, 102),
    "radial_iw2": ((24, 8, 9), (40, 8, 9), 2, 103),
}


def remesh_input(shape, seed):
    """Three complex fields of the given shape, real and imaginary parts uniform in [-1, 1)."""
    rng = SplitMix64(seed)
    n = int(np.prod(shape))
    vals = np.array([2.0 * rng.uniform() - 1.0 for _ in range(6 * n)])
    return [(vals[2 * n * c:2 * n * (c + 1):2] + 1j * vals[2 * n * c + 1:2 * n * (c + 1):2]).reshape(shape)
            for c in range(3)]


def make_remesh(outdir):
    fx = {}
    for name, (old, new, iw, seed) in REMESH_CASES.items():
        out = build_ref.run_remesh(old, new, iw, remesh_input(old, seed))
        fx[name] = np.stack(out)
        print("remesh", name, old, "->", new, "iw", iw, flush=True)
    np.savez_compressed(os.path.join(outdir, "remesh.npz"), **fx)


IO_FILES = ("io_friction.txt", "io_qcross.txt", "io_ucross.txt", "io_meanpr.txt")


def make_io(outdir, cfg="s2", nsteps=100):
    amp, seed = RUNS[cfg][:2]
    NR, NT, NZ, LZexpr, Re, dt = build_ref.CONFIGS[cfg]
    LZ = eval(LZexpr.replace("PI2", repr(PI2)))
    init_dir = os.path.join(tempfile.mkdtemp(prefix="nsp_golden_"), cfg + "_init")
    write_state(seeded_field(NR, NT, NZ, LZ, amp, seed), init_dir)
    rundir = build_ref.run(cfg, "io", init_dir, nsteps, nsteps_build=nsteps)
    dst = os.path.join(outdir, "io_" + cfg)
    os.makedirs(dst, exist_ok=True)
    for f in IO_FILES:
        shutil.copy2(os.path.join(rundir, f), os.path.join(dst, f))
    shutil.rmtree(init_dir)
    print("io", cfg, sorted(os.listdir(dst)), flush=True)


def main():
    outdir = os.path.abspath(sys.argv[1])
    cfgs = sys.argv[2:] or ["s2", "c0", "c1"]
    os.makedirs(outdir, exist_ok=True)
    summary = {}
    if "remesh" in cfgs:
        make_remesh(outdir)
        cfgs = [c for c in cfgs if c != "remesh"]
        if not cfgs:
            return
    if "io_s2" in cfgs:
        make_io(outdir)
        cfgs = [c for c in cfgs if c != "io_s2"]
        if not cfgs:
            return
    for cfg in cfgs:
        amp, seed, nsteps, snaps, full = RUNS[cfg]
        NR, NT, NZ, LZexpr, Re, dt = build_ref.CONFIGS[cfg]
        LZ = eval(LZexpr.replace("PI2", repr(PI2)))
        u0 = seeded_field(NR, NT, NZ, LZ, amp, seed)
        init_dir = os.path.join(tempfile.mkdtemp(prefix="nsp_golden_"), cfg + "_init")
        write_state(u0, init_dir)
        rundir = build_ref.run(cfg, "trace", init_dir, nsteps, snaps=snaps)
        iters = np.loadtxt(os.path.join(rundir, "iters.txt"), dtype=np.int64).reshape(-1, 2)[:, 1]
        fx = {"iters": iters, "init": np.stack(u0) if full else np.zeros(0),
              "params": np.array([NR, NT, NZ, Re, dt, LZ, amp, seed, nsteps], dtype=np.float64)}
        for s in snaps:
            u = read_state(rundir, (NR, NT, NZ), suffix="_%d" % s)
            if full:
                fx["u_%d" % s] = np.stack(u)
            else:
                for k, v in reduce_field(u, seed).items():
                    fx["%s_%d" % (k, s)] = v
        # drop the raw snapshots of every step
        for f in os.listdir(rundir):
            if f.endswith(".bin") and not f.endswith("_s.bin"):
                os.remove(os.path.join(rundir, f))
        np.savez_compressed(os.path.join(outdir, "ref_%s.npz" % cfg), **fx)
        summary[cfg] = {"iters": iters.tolist(), "snaps": snaps}
        shutil.rmtree(init_dir)
        print(cfg, "iters", iters.tolist(), flush=True)
    with open(os.path.join(outdir, "golden_summary.json"), "w") as fh:
        json.dump(summary, fh)


if __name__ == "__main__":
    main()
