"""Benchmark of the GB300 WCSPH hot path on config 2: the 2M-particle 3D jet in crossflow.

Workload (fjsph_gb300.cases.jet_crossflow_live, seeded synthetic inputs): a live inlet at dx =
50 um feeds the jet through a ghost-walled 2 mm pipe -- BACK particles crossing the inlet plane
insert new BUFFER particles, particles leaving the 20D x 20D x 10D domain downstream are deleted,
insertions stop at 2M live particles -- into a 50 m/s crossflow with a 1/7-power-law boundary
layer of thickness 5 mm (the analytic air field, settings asource FJSPH_POWER_LAW); pairwise
surface tension and the Gissler aero closure.  The run starts from the jet already emitted (the
bent column and droplets) at ~1.95M particles.

One step = one Integrator::integrate (src/Integration.cpp:233): CFL time step, neighbour searches,
the pre-passes, a Runge-Kutta-4 step with its four residual evaluations, and update_data
(insertion and deletion).  Particle-steps count the fluid particles each step processed.  The
state is resident in HBM when the timed region starts and is larger than the 129 MB L2, so no
flush is needed between steps.

The headline form is FP32 split precision with the learned aerodynamic closure; its network is
trained untimed before the run on the GPU from samples logged by seeded plain-closure runs of the
same workload (jet speed ~ U(5, 20) m/s, crossflow ~ U(30, 80) m/s).  The plain FP64 form and the
FP32 form with the plain closure are timed beside it from the same start.  Side sections: the
per-step error of the FP32 form against the FP64 oracle on a cut of the workload (`parity`),
config 0 (2D dam break, 2000 steps, GPU and the CPU restatement on all host cores), config 1 (3D
dam break, 16M fluid, FP32 against FP64 on identical states), config 4 (256 droplets), the air
sources and host set-up.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--n PARTICLES]

Prints one JSON line (rank 0).  `--impl reference` runs the CPU restatement of the reference
algorithm (the oracle; the reference itself cannot be built here) on the same workload, all host
cores, without loading the GPU library.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "particle-steps/s, 2M-particle jet: FP32+learned aero vs plain FP64, same GB300"
UNIT = "particle-steps/s"
WORKLOAD = "jet_in_crossflow_3d_live_inlet"
JET_SPEED = 10.0  # m/s, the inlet velocity of config 2


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=6)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=2_000_000, help="particle cap of the live jet (max_points)")
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--fp64-steps", type=int, default=2, help="steps of the plain FP64 form timed beside (0 = skip)")
    ap.add_argument("--e2e-steps", type=int, default=4)
    ap.add_argument("--vlm-points", type=int, default=1 << 20, help="points of the VLM air-source timing (0 = skip)")
    ap.add_argument("--mesh-cell", type=float, default=8e-4,
                    help="cube edge of the tetrahedral air mesh over the jet (0 = skip)")
    ap.add_argument("--setup-particles", type=int, default=2_000_000,
                    help="particles of the block-file setup timing (0 = skip)")
    ap.add_argument("--cpu-sample", type=int, default=110_000, help="fluid particles in the CPU baseline cut")
    ap.add_argument("--cpu-steps", type=int, default=2, help="oracle steps on the cut (baseline and parity)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--closure", default="learned", choices=["learned", "plain"])
    ap.add_argument("--train-samples", type=int, default=5_000_000)
    ap.add_argument("--train-jets", type=int, default=10, help="seeded jets the samples are logged from")
    ap.add_argument("--train-epochs", type=int, default=12)
    ap.add_argument("--closure-weights", default="", help="load trained weights from this .npy (skip training)")
    ap.add_argument("--save-weights", default="", help="save the trained weights to this .npy")
    ap.add_argument("--plain-steps", type=int, default=2, help="steps of the FP32 form with the plain closure")
    ap.add_argument("--drops", type=int, default=256, help="droplets of the batched workload (0 = skip)")
    ap.add_argument("--drop-steps", type=int, default=10)
    ap.add_argument("--drop-steps-fp64", type=int, default=3)
    ap.add_argument("--drop-long", type=int, default=3000, help="steps of the long FP32 droplet run (0 = skip)")
    ap.add_argument("--drop-sample", type=int, default=16, help="droplets timed alone for the per-droplet times")
    ap.add_argument("--config0-steps", type=int, default=2000, help="2D dam-break steps (0 = skip)")
    ap.add_argument("--no-config0-cpu", action="store_true")
    ap.add_argument("--config1-dx", type=float, default=0.003, help="spacing of the 3D dam break (0 = skip)")
    ap.add_argument("--config1-steps", type=int, default=3, help="timed FP32 steps of the 3D dam break")
    ap.add_argument("--config1-long", type=int, default=0, help="a long FP32 run of the 3D dam break (steps)")
    ap.add_argument("--pairs", default="lists", choices=["lists", "tiles"],
                    help="pair sweeps of the FP32 form: pair lists or shared-memory tiles (residual)")
    ap.add_argument("--no-tune", action="store_true")
    ap.add_argument("--order", default="auto", choices=["auto", "grid", "sm"],
                    help="work order of the FP32 residual on the jet: the autotuner's choice, grid or SM-local")
    return ap.parse_args()


# ---------------------------------------------------------------------------------------------

class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm = [float(r[1]) for r in self.rows if len(r) > 8 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 8 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            if len(r) > 8:
                for k, nm in enumerate(names):
                    if "Active" in r[5 + k] and "Not" not in r[5 + k]:
                        reasons.add(nm)
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def run_vlm(args):
    """Vortex-lattice air source (the Examples/VLM wing, 1400 horseshoes) evaluated at seeded points
    around the wing: the split-precision form at args.vlm_points points, the FP64 form at 1/16 of
    them; kernel time from the air_source profile section, setup (panels, influence matrix, LU)
    on the host timed beside it."""
    import numpy as np
    from fjsph_gb300 import _cdefs as d, cases
    from fjsph_gb300._lib import lib
    from fjsph_gb300.api import Context
    c = cases.droplet_3d(diam=6e-4, dx=1e-4)
    rng = np.random.Generator(np.random.PCG64(5))
    n = args.vlm_points
    pts = np.column_stack([rng.uniform(-10, 40, n), rng.uniform(-30, 30, n), rng.uniform(-6, 6, n)])
    out = {"wing": "Examples/VLM (50 x 14 panels per side, sweep 32.5 deg, taper 0.6, 20 deg flap)",
           "points": "uniform in [-10, 40] x [-30, 30] x [-6, 6] m around the wing"}
    for form, prec, m in (("fp32", d.PREC_MIXED, n), ("fp64", d.PREC_FP64, max(n // 16, 1024))):
        s = c.settings.copy()
        for k in range(3):
            s.v_inf[k] = VLM_VINF[k]
        s.asource = d.VLM_INFL
        s.precision = prec
        ctx = Context(s, c.state.n + 64, c.blocks, c.inlets)
        ctx.set_states(c.state, c.state)
        v = d.Vlm()
        lib().fjsph_vlm_defaults(v)
        for k, val in VLM_WING.items():
            setattr(v, k, val)
        t0 = time.perf_counter()
        npan = ctx.vlm_setup(v)
        setup_s = time.perf_counter() - t0
        p = pts[:m]
        ctx.vlm_velocity(p[:4096])
        ctx.profile(True)
        ctx.profile_read()
        reps = 3
        for _ in range(reps):
            ctx.vlm_velocity(p)
        ms = ctx.profile_read()["air_source"][0] / reps
        ctx.profile(False)
        out[form] = {"points": m, "panels": npan, "kernel_ms": round(ms, 4), "evaluations_per_s": m / (ms / 1e3),
                     "panel_interactions_per_s": m * npan / (ms / 1e3), "setup_s": round(setup_s, 3)}
        ctx.close()
    return out


def run_case_setup(args):
    """Init_Particles from block files on the host (fjsph_gb300.geometry over the C ABI): a cube
    of water on a three-layer floor plane, sized for args.setup_particles, read from bmap text,
    checked, generated, culled against the floor and laid out; then uploaded once."""
    from fjsph_gb300.api import Context
    from fjsph_gb300.geometry import Geometry
    from fjsph_gb300.settings import defaults, derive
    side = 1.0
    dx = side / max(round(args.setup_particles ** (1.0 / 3.0)), 2)
    s = defaults(3)
    s.particle_step = dx
    derive(s)
    w = 3 * dx
    bound = (f"Name: Floor\nShape: Plane\nStart coordinate: {-w},0,{-w}\nRight coordinate: {side + w},0,{-w}\n"
             f"End coordinate: {side + w},0,{side + w}\nWall radial particle count: 3\nblock end\n")
    fluid = f"Name: Water\nShape: Cube\nStart coordinate: 0,0,0\nEnd coordinate: {side},{side},{side}\nblock end\n"
    t0 = time.perf_counter()
    g = Geometry(s)
    g.read_text(bound, False)
    g.read_text(fluid, True)
    g.build()
    t1 = time.perf_counter()
    st, blocks = g.state(), g.blocks()
    t2 = time.perf_counter()
    ctx = Context(s, st.n + 64, blocks, [])
    ctx.set_states(st, st)
    ctx.event_record(0)
    ctx.event_record(1)
    ctx.event_elapsed(0, 1)  # waits for the stream
    t3 = time.perf_counter()
    info = g.block_info()
    g.close()
    ctx.close()
    return {"case": "water cube on a 3-layer floor plane (bmap text)", "particles": st.n,
            "generated": int(sum(b["generated"] for b in info)), "dx": dx,
            "build_s": round(t1 - t0, 3), "state_s": round(t2 - t1, 3), "upload_s": round(t3 - t2, 3),
            "particles_per_s": st.n / (t1 - t0), "where": "host (one thread), then one upload"}


def run_mesh(args, case):
    """The mesh-cell air source on the jet: a tetrahedral mesh over the jet's bounding box carries
    a seeded air solution; FindCell (containment of every free surface particle, in place of the
    uniform aero velocity) timed alone, and whole steps of the FP32 form with the plain closure."""
    import numpy as np
    from fjsph_gb300 import _cdefs as d
    from fjsph_gb300.api import Context
    from fjsph_gb300.mesh import tet_mesh_3d
    st = case.state
    lo, hi = st.xi.min(axis=0) - 1e-4, st.xi.max(axis=0) + 1e-4
    h = args.mesh_cell
    n = tuple(int(max(1, np.ceil((hi[k] - lo[k]) / h))) for k in range(3))
    t0 = time.perf_counter()
    mesh = tet_mesh_3d(lo=tuple(lo), hi=tuple(lo + np.array(n) * h), n=n, u0=50.0, seed=3)
    build_s = time.perf_counter() - t0
    s = case.settings.copy()
    s.asource = d.MESH_INFL
    s.precision = d.PREC_MIXED
    s.aero_closure = d.CLOSURE_PLAIN
    ctx = Context(s, s.max_points + 1024, case.blocks, case.inlets)
    t0 = time.perf_counter()
    ctx.mesh_set(mesh)
    set_s = time.perf_counter() - t0
    ctx.set_states(st, st)
    ctx.integrate()
    ctx.update_neighbours()
    ctx.dSPH_PreStep()
    reps = 5
    ctx.get_aero_velocity()  # every active particle located once (later calls start from its cell)
    ctx.event_record(2)
    for _ in range(reps):
        ctx.get_aero_velocity()
    ctx.event_record(3)
    find_ms = ctx.event_elapsed(2, 3) / reps
    got = ctx.download()
    active = int(np.count_nonzero(got.cellID >= 0))
    ctx.close()

    def steps_ms(settings, with_mesh):
        """whole steps after three warm-up steps, this context alone on the GPU"""
        cx = Context(settings, settings.max_points + 1024, case.blocks, case.inlets)
        if with_mesh:
            cx.mesh_set(mesh)
        cx.set_states(st, st)
        for _ in range(3):
            cx.integrate()
        cx.event_record(4)
        for _ in range(3):
            cx.integrate()
        cx.event_record(5)
        ms = cx.event_elapsed(4, 5) / 3
        cx.close()
        return ms

    step_ms = steps_ms(s, True)
    s_uniform = s.copy()
    s_uniform.asource = d.CONST_VEL
    uniform_ms = steps_ms(s_uniform, False)
    return {"mesh": f"{mesh.n_cells} tetrahedra ({n[0]} x {n[1]} x {n[2]} cubes of {h * 1e3:.2f} mm, six each)",
            "particles": st.n, "located": active, "find_cell_ms": round(find_ms, 4),
            "located_per_s": active / (find_ms / 1e3) if find_ms > 0 else None,
            "fp32_step_ms": round(step_ms, 3), "particle_steps_per_s": case.n_fluid / (step_ms / 1e3),
            "fp32_step_ms_uniform_source": round(uniform_ms, 3),
            "mesh_build_s": round(build_s, 2), "mesh_set_s": round(set_s, 3)}


def pinned_state(st):
    """Copy of st whose arrays live in page-locked host memory (torch is used only to allocate)."""
    from fjsph_gb300.state import ALL_FIELDS
    out = st.copy()
    out._pinned = False
    try:
        import torch
        if torch.cuda.is_available():
            for f in ALL_FIELDS:
                a = getattr(st, f)
                t = torch.empty(a.shape, dtype=getattr(torch, str(a.dtype)), pin_memory=True)
                arr = t.numpy()
                arr[...] = a
                setattr(out, f, arr)
                out.__dict__.setdefault("_keep", []).append(t)
            out._pinned = True
    except Exception:
        pass
    return out


def download_into(ctx, st, fields=None) -> None:
    from fjsph_gb300 import _cdefs as d
    ctx.download(d.PNP1, fields=fields, out=st)


def state_bytes(st, fields=None) -> int:
    from fjsph_gb300.state import ALL_FIELDS
    return int(sum(getattr(st, f).nbytes for f in (fields or ALL_FIELDS)))


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def reduce_max(ws, x: float) -> float:
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"  # gloo ranks reduce on the host
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return json.loads(p.read_text())
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "fallback": True}


# ---------------------------------------------------------------------------------------------


def resid_bytes_per_particle(s) -> int:
    """Algorithmic bytes of one residual evaluation per fluid particle.

    Each logical field is counted once per launch; neighbour re-reads and the pair list do not
    count.  FP64 form (8 B words): x 3, search x 3, v 3, rho, p, m, aVisc 3, deltaD, cellV 3,
    cellP, cellRho, lam_nb, woccl (8 B each), cellID, CSR offset (8 B), b, surfzone (4 B); ALE adds
    vPert 3, NOFROZEN gradRho 3.  Writes acc 3, Af 3, Rrho.
    FP32 split-precision form: x and v as an FP32 high part and a bf16 low part (6 B per
    component), rho, p / rho^2 with the type flags and volume at 4 B; aVisc 3 and deltaD (FP64
    state), CSR offset and cellID (8 B); the closure reads
    cellV 3, cellP, cellRho, m, lam_nb, woccl (8 B), the learned closure also the four occlusion
    inputs, the normal and lambda (4 B each).  Writes acc 3, Af 3, Rrho at 8 B.
    """
    from fjsph_gb300 import _cdefs as d
    D = s.dim
    if s.precision == d.PREC_MIXED:
        b = 6 * D * 2 + 4 * 3                      # x, v (FP32 high, bf16 low), rho, p/rho^2, volume
        b += 8 * (D + 1) + 8 * 2                   # aVisc, deltaD, CSR offset, cellID
        b += 8 * (D + 5)                           # cellV, cellP, cellRho, m, lam_nb, woccl
        if s.aero_closure == d.CLOSURE_LEARNED:
            b += 4 * (4 + D + 1)                   # occlusion inputs, normal, lambda
        if s.variant & d.VAR_ALE:
            b += 4 * D
        if s.variant & d.VAR_NOFROZEN:
            b += 4 * D
        return b + 8 * (2 * D + 1)
    r8 = 3 * D + 3 + 3 + D + 1 + D + 2 + 2 + 2 + 1
    if s.variant & d.VAR_ALE:
        r8 += D
    if s.variant & d.VAR_NOFROZEN:
        r8 += D
    w8 = 2 * D + 1
    return 8 * (r8 + w8) + 4 * 2


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


# DRAM bytes (read + write) per fluid particle of one residual launch, from one ncu capture
# (dram__bytes_read.sum + dram__bytes_write.sum / fluid particles); scaled to the benchmark's
# particle count (traffic grows with the particle and pair counts).
RESID_TRAFFIC_PER_PARTICLE = {"fp64": 42.100e9 * 7.8264e-3 / 547_607, "mixed": (469.264e6 + 55.326e6) / 547_607}
TRAFFIC_SOURCE = {"fp64": "ncu capture of k_resid on the 570k-particle live jet (dram__bytes.sum.per_second x "
                          "gpu__time_duration.sum), scaled by fluid particles",
                  "mixed": "ncu capture of k_m_resid (plain closure, grid order) on the 570k-particle live jet, "
                           "scaled by fluid particles"}
# Both fractions of the split-precision residual from the same capture (pct of peak, elapsed): the
# memory side and the compute pipes, and the unit that binds.
RESID_PIPES_MIXED = {"dram": 0.167, "l1tex": 0.713, "lts": 0.715, "fp32_fma": 0.323, "alu": 0.236, "xu": 0.136,
                     "fp64": 0.123, "tensor": 0.0, "binding": "l1tex/lts: three 16-byte neighbour gathers per pair",
                     "source": "ncu capture of k_m_resid (plain closure, grid order) on the 570k-particle live jet"}

# Examples/VLM: a 22.3 m half-span, 8.5 m chord wing, sweep 32.5 deg, taper 0.6, 20 deg flap
VLM_WING = dict(span=22.275, chord=8.491, panels_span=50, panels_chord=14, aoa_deg=5.0, sweep_deg=32.5, taper=0.6,
                flap_start=3, flap_width=24, flap_depth=6, flap_deg=20.0)
VLM_VINF = (89.69, 0.0, 7.8466)


def train_closure(args, log):
    """Untimed: log samples from seeded plain-closure runs of the workload and train the network
    on the GPU."""
    import numpy as np
    from fjsph_gb300 import closure as cl
    info = {}
    if args.closure_weights and Path(args.closure_weights).exists():
        info["weights"] = f"loaded from {args.closure_weights}"
        return np.load(args.closure_weights).astype(np.float32), info
    t0 = time.perf_counter()
    specs = cl.jet_specs(args.train_jets, 800_000, seed=2024, live=True)
    X, T = cl.collect_samples(specs, args.train_samples, steps=8)
    t1 = time.perf_counter()
    p0 = cl.init_params(X, T, seed=7)
    p, loss = cl.train(p0, X, T, epochs=args.train_epochs, batch=4096, lr=2e-3, seed=8)
    t2 = time.perf_counter()
    info.update(samples=int(len(X)), jets=len(specs), log_s=round(t1 - t0, 2), train_s=round(t2 - t1, 2),
                epochs=args.train_epochs, final_loss=loss,
                jet_speeds=[round(sp.jet_speed, 2) for sp in specs], air_speeds=[round(sp.air_speed, 2) for sp in specs])
    if args.save_weights:
        np.save(args.save_weights, p)
    log(f"closure trained: {info}")
    return p, info


def make_case(n_cap: int, precision: str, closure: str = "plain"):
    from fjsph_gb300 import cases, _cdefs as d
    c = cases.jet_crossflow_live(n_target=n_cap, cap=n_cap, jet_speed=JET_SPEED)
    if precision == "mixed":
        c.settings.precision = d.PREC_MIXED
        if closure == "learned":
            c.settings.aero_closure = d.CLOSURE_LEARNED
    return c


def new_ctx(settings, c, state=None):
    """A context for case c under `settings` (capacity: the insertion cap for a case with inlets,
    else the particles), with the case's inlet tables and analytic air field, holding `state`
    (default: the case's start)."""
    from fjsph_gb300 import _cdefs as d
    from fjsph_gb300.api import Context
    st = state if state is not None else c.state
    cap = max(settings.max_points, st.n) + 1024 if c.inlets else st.n + 1024  # insertions need room
    ctx = Context(settings, cap, c.blocks, c.inlets)
    if settings.asource == d.POWER_LAW and c.power_law_params:
        ctx.air_power_law(*c.power_law_params)
    ctx.set_states(st, st)
    return ctx


def counted_steps(ctx, steps: int, nb: int) -> tuple[float, int]:
    """steps integrate() calls between two events on the context's stream; returns the device
    time (ms) and the fluid particle-steps processed (the count changes with insertion and
    deletion: each step counts the particles it started with)."""
    ps = 0
    ctx.event_record(0)
    for _ in range(steps):
        ps += ctx.particle_count() - nb
        ctx.integrate()
    ctx.event_record(1)
    return ctx.event_elapsed(0, 1), ps


def prefix_state(big, n: int):
    """The first n particles of a (pinned) state, as a state sharing its memory."""
    from fjsph_gb300.state import ALL_FIELDS, SPHState
    out = SPHState.__new__(SPHState)
    out.n, out.dim = int(n), big.dim
    for f in ALL_FIELDS:
        setattr(out, f, getattr(big, f)[:n])
    out._pinned = getattr(big, "_pinned", False)
    return out




def pinned_buffer(n: int, dim: int):
    """A zeroed state of n particles in page-locked host memory (torch only allocates)."""
    from fjsph_gb300.state import SPHState
    return pinned_state(SPHState(n, dim))


def roofline(s, prof, nf_mean: float, peaks: dict, learned: bool, tiles: bool = False) -> dict:
    """The residual (the dominant kernel): algorithmic bytes per fluid particle x the fluid
    particles of a launch, over the launch's mean device time from the profile events."""
    from fjsph_gb300 import _cdefs as d
    r_ms, r_cnt = prof["residual"]
    bpp = resid_bytes_per_particle(s)
    per_launch = r_ms / max(r_cnt, 1) / 1e3
    achieved = bpp * nf_mean / per_launch / 1e9
    tkey = "fp64" if s.precision == d.PREC_FP64 else ("mixed" if not tiles else None)
    traffic = round(RESID_TRAFFIC_PER_PARTICLE[tkey] * nf_mean) if tkey else None
    peak = peaks.get("hbm_gbs", 6800.0)
    return {"bound": "hbm", "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "traffic": traffic,
            "traffic_source": TRAFFIC_SOURCE.get(tkey),
            "kernel": (("k_t_resid" if tiles else "k_m_resid") if s.precision == d.PREC_MIXED else "k_resid")
            + " (get_acc_and_Rrho)",
            "launch_ms": round(per_launch * 1e3, 3), "bytes_per_launch": round(bpp * nf_mean),
            "bytes_per_particle": bpp, "peak_source": "measured" if not peaks.get("fallback") else "fallback",
            "pipes_ncu": RESID_PIPES_MIXED if tkey == "mixed" else None}


def run_ours(args, ws, rank, local):
    import numpy as np
    from fjsph_gb300 import _cdefs as d
    from fjsph_gb300.state import STEP_FIELDS

    learned = args.precision == "mixed" and args.closure == "learned"
    weights, closure_info = (train_closure(args, lambda m: print(m, file=sys.stderr)) if learned else (None, None))
    c = make_case(args.n, args.precision, args.closure)
    s = c.settings
    nb = c.state.n - c.n_fluid
    ctx = new_ctx(s, c)
    if args.pairs == "tiles":
        ctx.set_pair_mode(d.PAIRS_TILES)
    if learned:
        ctx.closure_set_weights(weights, 0.05)
    for _ in range(args.warmup):
        ctx.integrate()
    tune = ctx.autotune(3) if s.precision == d.PREC_MIXED and not args.no_tune else None
    if s.precision == d.PREC_MIXED and args.order != "auto":
        ctx.set_sweep_order(d.ORDER_SM if args.order == "sm" else d.ORDER_GRID)
    if tune or args.order != "auto":
        ctx.integrate()  # one more warm-up step under the chosen configuration
    order = ("sm" if ctx.sweep_order() == d.ORDER_SM else "grid") if s.precision == d.PREC_MIXED else None
    barrier(ws)
    clocks = Clocks(local)
    clocks.start()
    ctx.profile(True)
    ctx.launch_stats(reset=True)
    ins0, del0 = ctx.update_counts()
    t_sim0 = ctx.settings.current_time
    ms, ps = counted_steps(ctx, args.steps, nb)
    launches = ctx.launch_stats()
    ins1, del1 = ctx.update_counts()
    t_sim1 = ctx.settings.current_time
    n_pairs = ctx.update_neighbours()  # pairs of the last search (outside the timed region)
    prof = ctx.profile_read()
    ctx.profile(False)
    clk = clocks.stop()
    ms = reduce_max(ws, ms)
    value = ps * ws / (ms / 1e3)
    nf_mean = ps / args.steps
    rep = ctx.step_report()
    roof = roofline(s, prof, nf_mean, measured_peaks(), learned, args.pairs == "tiles")
    live = {"particles_at_start": int(c.state.n), "particles_at_end": int(ctx.particle_count()),
            "inserted_in_timed_steps": int(ins1 - ins0), "deleted_in_timed_steps": int(del1 - del0),
            "inserted_total": int(ins1), "deleted_total": int(del1), "cap": int(s.max_points),
            "mean_fluid_per_step": round(nf_mean, 1),
            "simulated_us_in_timed_steps": round((t_sim1 - t_sim0) * 1e6, 3),
            "insertion_interval_us": round(s.particle_step / JET_SPEED * 1e6, 3),
            "note": "a column inserts a layer each time its BACK particle has travelled one dx at the jet "
                    "speed (src/shapes/inlet.cpp:578-640); the time step is set by the inlet's deepest "
                    "buffer layer, as upstream, whose find_timestep includes the buffer"}

    # the learned closure judged against the plain one on the state the timed steps reached
    if learned:
        ctx.closure_arm(d.CLOSURE_ARM_JUDGE)
        ctx.integrate()
        rep_c = ctx.closure_report()
        closure_info.update(judge_rel_rms=rep_c["last_rel_rms"], judge_particles=rep_c["judged_particles"],
                            judged=rep_c["judged"], fallback=bool(rep_c["fallback"]),
                            learned_active=bool(rep_c["learned_active"]),
                            judge_interval_steps=s.learned_judge_interval)

    # end to end through the public API with host buffers in pinned memory: every step uploads the
    # step's input fields (FJSPH_STEP_FIELDS, as both pn and pnp1) and downloads the same fields
    # of the new state; the particle count follows the inlet and the deletion plane
    e2e = None
    if args.e2e_steps > 0:
        host = pinned_buffer(s.max_points + 1024, s.dim)
        ctx.download(d.PNP1, out=prefix_state(host, ctx.particle_count()))
        # one untimed call first: it sizes the call's staging buffers and creates its streams
        ctx.step_host(prefix_state(host, ctx.particle_count()), host, fields=STEP_FIELDS)
        h2d = d2h = 0
        ps_e = 0
        ctx.event_record(2)
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            n = ctx.particle_count()
            st = prefix_state(host, n)
            # fjsph_step_host: pn = pnp1 = st, one step, pnp1 back into the same pinned arrays
            n2 = ctx.step_host(st, host, fields=STEP_FIELDS)
            h2d += state_bytes(st, STEP_FIELDS)
            d2h += state_bytes(prefix_state(host, n2), STEP_FIELDS)
            ps_e += n - nb
        ctx.event_record(3)
        e2e_ms = ctx.event_elapsed(2, 3)
        wall = time.perf_counter() - t0
        e2e_ms = reduce_max(ws, max(e2e_ms, wall * 1e3))
        e2e = {"value": ps_e * ws / (e2e_ms / 1e3), "unit": UNIT,
               "h2d_bytes_per_step": h2d // args.e2e_steps, "d2h_bytes_per_step": d2h // args.e2e_steps,
               "pinned": host._pinned,
               "fields": "FJSPH_STEP_FIELDS (the state a step reads; the rest is recomputed inside it)",
               "call": "fjsph_step_host: upload as pn and pnp1, one step, download; the fields a step first "
                       "reads after its first neighbour search travel in while that search runs, the fields "
                       "final after the second search's pre-passes travel out during the last stages"}
    ctx.close()

    def other_form(settings, steps):
        cx = new_ctx(settings, c)
        cx.integrate()
        cx.profile(True)
        msx, psx = counted_steps(cx, steps, nb)
        msx = reduce_max(ws, msx)
        pp = cx.profile_read()
        cx.close()
        return {"value": psx * ws / (msx / 1e3), "ms_per_step": msx / steps, "steps": steps,
                "residual_ms_per_launch": round(pp["residual"][0] / max(pp["residual"][1], 1), 4)}

    plain = None
    if learned and args.plain_steps > 0:
        sp_ = s.copy()
        sp_.aero_closure = d.CLOSURE_PLAIN
        plain = other_form(sp_, args.plain_steps)
    fp64 = None
    if args.fp64_steps > 0 and s.precision != d.PREC_FP64:
        s64 = s.copy()
        s64.precision = d.PREC_FP64
        s64.aero_closure = d.CLOSURE_PLAIN
        fp64 = other_form(s64, args.fp64_steps)
    return dict(value=value, ms=ms, nf=c.n_fluid, n=c.state.n, roof=roof, e2e=e2e, clocks=clk, launches=launches,
                fp64=fp64, prof={k: [round(v[0], 3), v[1]] for k, v in prof.items() if v[1]}, rep=rep, settings=s,
                case=c, plain=plain, closure=closure_info, pairs=n_pairs, tune=tune, weights=weights, live=live,
                ps=ps, order=order)


def _rel_rms(a, b) -> float:
    import numpy as np
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    den = float(np.sqrt(np.mean(b * b))) if b.size else 0.0
    return float(np.sqrt(np.mean((a - b) ** 2)) / den) if den > 0 else 0.0


def run_cpu_parity(args, c, threads: int):
    """The CPU restatement (oracle, FP64, OpenMP on all host cores) on a contiguous cut of the
    workload -- the cpu_baseline timing -- and, on the same cut and states, the error of the FP32
    form against it: the residual on the oracle's pre-pass outputs, then each timed oracle step
    against one FP32 step from the same state (both time levels)."""
    import dataclasses
    import numpy as np
    from fjsph_gb300 import _cdefs as d
    from fjsph_gb300 import cases
    from oracle.pyoracle import Oracle, set_threads
    set_threads(threads)
    cc = cases.cut(c, args.cpu_sample)
    s64 = cc.settings.copy()
    s64.precision = d.PREC_FP64
    s64.aero_closure = d.CLOSURE_PLAIN
    cc = dataclasses.replace(cc, settings=s64)
    s32 = s64.copy()
    s32.precision = d.PREC_MIXED
    nb = sum(b.second - b.first for b in cc.blocks if not b.is_fluid)
    nf = cc.state.n - nb

    def oracle():
        o = Oracle(cc.settings, cc.blocks)
        if cc.power_law_params:
            o.air_power_law(*cc.power_law_params)
        o.set_states(cc.state, cc.state)
        return o

    # the residual alone on the oracle's pre-pass outputs
    o = oracle()
    o.update_neighbours()
    npd = o.dSPH_PreStep()
    o.get_aero_velocity()
    o.Detect_Surface()
    o.dissipation_terms()
    o.Boundary_Ghost()
    prepared = o.download()
    o.get_acc_and_Rrho(npd)
    ref = o.download()
    o.close()
    g_ctx = new_ctx(s32, cc, prepared)
    g_ctx.update_neighbours()
    g_ctx.get_acc_and_Rrho(npd)
    g = g_ctx.download()
    g_ctx.close()
    sl = slice(nb, None)
    resid = {"Rrho": _rel_rms(g.Rrho[sl], ref.Rrho[sl]), "acc": _rel_rms(g.acc[sl], ref.acc[sl]),
             "Af": _rel_rms(g.Af[sl], ref.Af[sl])}
    # timed oracle steps (the baseline), each compared with one FP32 step from the same state
    o = oracle()
    steps, t_cpu, e_x, e_rho = [], 0.0, [], []
    for k in range(args.cpu_steps):
        pn, pnp1, sk = o.download(d.PN), o.download(d.PNP1), o.settings
        t0 = time.perf_counter()
        o.integrate()
        t_cpu += time.perf_counter() - t0
        r = o.download()
        sk.precision = d.PREC_MIXED
        gx = new_ctx(sk, cc, pnp1)
        gx.upload(d.PN, pn)
        gx.integrate()
        gs = gx.download()
        gx.close()
        e_x.append(_rel_rms(gs.xi[sl] - pnp1.xi[sl], r.xi[sl] - pnp1.xi[sl]))
        e_rho.append(_rel_rms(gs.rho[sl] - pnp1.rho[sl], r.rho[sl] - pnp1.rho[sl]))
    o.close()
    cpu = {"value": nf * args.cpu_steps / t_cpu, "unit": UNIT, "cores": threads, "kind": "port",
           "sample": f"{args.cpu_steps} Integrator::integrate steps of the {nf} fluid particles nearest the pipe "
                     f"exit cut from the workload (CPU restatement, {t_cpu:.1f} s)"}
    parity = {"reference": "oracle (FP64 CPU restatement)", "cut_fluid_particles": nf, "form": "FP32, plain closure",
              "residual_rel_rms": resid, "step_displacement_rel_rms": e_x, "step_density_change_rel_rms": e_rho,
              "targets": {"Rrho": 1e-5, "acc": 1e-3}}
    return cpu, parity


def run_config0(args, threads: int, rank: int):
    """Config 0: the 2D dam break (20,000 fluid particles, RK4, CFL 0.2) for its full step count on
    the GPU (FP64 and FP32 forms) and on the host cores (the CPU restatement)."""
    import numpy as np
    from fjsph_gb300 import _cdefs as d
    from fjsph_gb300 import cases
    steps = args.config0_steps
    c = cases.dam_break_2d()
    nb = c.state.n - c.n_fluid
    out = {"case": "2D dam break: 1.0 x 2.0 m column, 4.0 x 3.0 m tank, dx 0.01, 3 wall layers, RK4, CFL 0.2",
           "particles": int(c.state.n), "fluid": int(c.n_fluid), "steps": steps}
    finals = {}
    for name, prec in (("gpu_fp64", d.PREC_FP64), ("gpu_fp32", d.PREC_MIXED)):
        s = c.settings.copy()
        s.precision = prec
        warm = new_ctx(s, c)  # first launches and allocations outside the timing
        for _ in range(3):
            warm.integrate()
        warm.close()
        ctx = new_ctx(s, c)
        pairs = ctx.update_neighbours()
        t0 = time.perf_counter()
        ms, ps = counted_steps(ctx, steps, nb)
        wall = time.perf_counter() - t0
        finals[name] = ctx.download()
        out[name] = {"value": ps / (ms / 1e3), "unit": UNIT, "wall_s": round(wall, 3),
                     "neighbour_pairs_per_s": pairs * steps / (ms / 1e3),
                     "sim_time_s": ctx.settings.current_time}
        ctx.close()
    # the same steps through a context holding the dam break as its one group: the step runs
    # without host round trips and replays as a CUDA graph (fjsph_integrate_groups)
    for name, prec in (("gpu_fp64_graph", d.PREC_FP64), ("gpu_fp32_graph", d.PREC_MIXED)):
        s = c.settings.copy()
        s.precision = prec
        for warm_up in (True, False):
            ctx = new_ctx(s, c)
            ctx.set_groups([0, c.state.n], [list(s.v_inf)])
            ctx.event_record(0)
            t0 = time.perf_counter()
            ctx.integrate_groups(3 if warm_up else steps, graph=True)
            ctx.event_record(1)
            wall = time.perf_counter() - t0
            if warm_up:
                ctx.close()
                continue
            ms = max(ctx.event_elapsed(0, 1), wall * 1e3)
            rep = ctx.group_report()
            finals[name] = ctx.download()
            out[name] = {"value": c.n_fluid * steps / (ms / 1e3), "unit": UNIT, "wall_s": round(wall, 3),
                         "sim_time_s": float(rep["time"][0]), "steps": int(rep["steps"][0]),
                         "launch": "fjsph_integrate_groups with one group: each step one CUDA-graph replay "
                                   "(captured on first use, inside the timing)"}
            ctx.close()
    if rank == 0 and not args.no_config0_cpu:
        from oracle.pyoracle import Oracle, set_threads
        set_threads(threads)
        o = Oracle(c.settings, c.blocks)
        o.set_states(c.state, c.state)
        pairs = o.update_neighbours()
        t0 = time.perf_counter()
        for _ in range(steps):
            o.integrate()
        wall = time.perf_counter() - t0
        r = o.download()
        out["cpu"] = {"value": c.n_fluid * steps / wall, "unit": UNIT, "cores": threads, "kind": "port",
                      "wall_s": round(wall, 2), "neighbour_pairs_per_s": pairs * steps / wall,
                      "sim_time_s": o.settings.current_time}
        sl = slice(nb, None)
        out["final_state_gpu_fp64_vs_cpu"] = {
            "x_rel_rms": _rel_rms(finals["gpu_fp64"].xi[sl], r.xi[sl]),
            "rho_rel_rms": _rel_rms(finals["gpu_fp64"].rho[sl], r.rho[sl])}
        for name in ("gpu_fp32", "gpu_fp64_graph", "gpu_fp32_graph"):
            out[f"final_state_{name}_vs_cpu"] = {
                "x_rel_rms": _rel_rms(finals[name].xi[sl], r.xi[sl]),
                "rho_rel_rms": _rel_rms(finals[name].rho[sl], r.rho[sl])}
        o.close()
    return out


def run_config1(args):
    """Config 1: the 3D dam break (0.6 x 0.6 x 1.2 m column, 1.6 x 0.6 x 1.2 m tank, dx 3 mm: ~16M
    fluid and ~2.1M wall particles, lattice jittered by +-0.01 dx, ALE shifting) on one GPU: FP32
    and FP64 forms timed, and one step of each from the identical start compared."""
    from fjsph_gb300 import _cdefs as d
    from fjsph_gb300 import cases
    t0 = time.perf_counter()
    c = cases.dam_break_3d(dx=args.config1_dx)
    build_s = time.perf_counter() - t0
    nb = c.state.n - c.n_fluid
    out = {"case": f"3D dam break, dx {args.config1_dx * 1e3:g} mm, ALE, jitter +-0.01 dx, RK4, CFL 0.2",
           "particles": int(c.state.n), "fluid": int(c.n_fluid), "build_s": round(build_s, 1)}
    fields = ["xi", "rho", "acc", "Rrho"]
    first = {}
    for name, prec, steps in (("fp32", d.PREC_MIXED, args.config1_steps), ("fp64", d.PREC_FP64, 1)):
        s = c.settings.copy()
        s.precision = prec
        ctx = new_ctx(s, c)
        ctx.integrate()
        first[name] = ctx.download(d.PNP1, fields=fields)
        tune = ctx.autotune(3)["chosen"] if prec == d.PREC_MIXED and not args.no_tune else None
        pairs = ctx.update_neighbours()
        ctx.profile(True)
        ms, ps = counted_steps(ctx, steps, nb)
        prof = ctx.profile_read()
        ctx.profile(False)
        out[name] = {"value": ps / (ms / 1e3), "unit": UNIT, "ms_per_step": ms / steps, "steps": steps,
                     "neighbour_pairs": int(pairs), "neighbour_pairs_per_s": pairs * steps / (ms / 1e3),
                     "passes_ms_per_step": {k: round(v[0] / steps, 3) for k, v in prof.items() if v[1]}}
        if tune:
            out[name]["autotune"] = tune
        if name == "fp32" and args.config1_long > 0:
            ms_l, ps_l = counted_steps(ctx, args.config1_long, nb)
            out["fp32_long"] = {"steps": args.config1_long, "value": ps_l / (ms_l / 1e3), "unit": UNIT,
                                "wall_s": round(ms_l / 1e3, 1), "sim_time_s": ctx.settings.current_time}
        ctx.close()
    sl = slice(nb, None)
    a, b = first["fp32"], first["fp64"]
    x0 = c.state.xi[sl]
    out["step_error_fp32_vs_fp64"] = {
        "displacement_rel_rms": _rel_rms(a.xi[sl] - x0, b.xi[sl] - x0),
        "density_change_rel_rms": _rel_rms(a.rho[sl] - c.state.rho[sl], b.rho[sl] - c.state.rho[sl]),
        "acc_rel_rms": _rel_rms(a.acc[sl], b.acc[sl]), "Rrho_rel_rms": _rel_rms(a.Rrho[sl], b.Rrho[sl]),
        "note": "one integrate step of each form from the identical start; the FP64 form is checked against "
                "the oracle on cuts (tests/test_gpu_scale.py)"}
    out["speedup_fp32_over_fp64"] = out["fp32"]["value"] / out["fp64"]["value"]
    return out


def run_droplets(args, ws, rank, weights):
    """Config 4: a batch of independent droplets in one context per GPU (droplets shared out over
    the ranks with no exchange), each step one CUDA-graph replay; plain FP64, FP32 with the plain
    closure and FP32 with the learned closure.  Per-droplet work: each droplet's share of the
    batch step by its neighbour pairs.  Rank 0 also times a sample of droplets alone (one context
    each) and runs the FP32 batch for the configuration's 3000 steps."""
    import numpy as np
    from fjsph_gb300 import _cdefs as d
    from fjsph_gb300 import cases
    from fjsph_gb300.api import Context
    full = cases.droplet_batch(n_drops=args.drops)
    ids = cases.shard_ids(len(full.counts), full.counts, rank, ws)
    b = full.subset(ids) if ws > 1 else full
    n = b.case.state.n
    total = full.case.state.n
    out = {"droplets": int(len(full.counts)), "particles": int(total), "counts_range": [int(full.counts.min()),
           int(full.counts.max())], "we_range": [round(float(full.we.min()), 1), round(float(full.we.max()), 1)],
           "sharding": f"{ws} rank(s), greedy particle balance, no collective but the final timing max",
           "config_steps": 3000, "forms": {},
           "launch": "each pass one launch over all droplets, a step one CUDA-graph replay (no persistent kernel)"}
    forms = [("fp64", d.PREC_FP64, d.CLOSURE_PLAIN, args.drop_steps_fp64),
             ("fp32_plain_closure", d.PREC_MIXED, d.CLOSURE_PLAIN, args.drop_steps),
             ("fp32_learned_closure", d.PREC_MIXED, d.CLOSURE_LEARNED, args.drop_steps)]
    long_form = None
    for name, prec, closure, steps in forms:
        if closure == d.CLOSURE_LEARNED and weights is None:
            continue
        s = b.case.settings.copy()
        s.precision = prec
        s.aero_closure = closure
        ctx = Context(s, n + 64, b.case.blocks)
        ctx.set_groups(b.first, b.v_inf)
        ctx.set_states(b.case.state, b.case.state)
        if closure == d.CLOSURE_LEARNED:
            ctx.closure_set_weights(weights, 0.05)
        tune = ctx.autotune(3)["chosen"] if prec == d.PREC_MIXED and not args.no_tune else None
        ctx.integrate_groups(2, graph=True)  # one ordinary step, then the graph capture
        barrier(ws)
        ctx.launch_stats(reset=True)
        ctx.event_record(0)
        ctx.integrate_groups(steps, graph=True)
        ctx.event_record(1)
        ms = reduce_max(ws, ctx.event_elapsed(0, 1))
        rep = ctx.group_report()
        ctx.update_neighbours()
        cnt = ctx.neighbour_counts().astype(np.float64)
        pairs_g = np.add.reduceat(cnt, b.first[:-1])
        work = (ms / steps) * pairs_g / pairs_g.sum()  # each droplet's share of the batch step
        out["forms"][name] = {"value": total * steps / (ms / 1e3), "unit": UNIT, "ms_per_step": ms / steps,
                              "steps": steps, "gpu_launches_per_step": ctx.launch_stats() / steps,
                              "graph": True, "autotune": tune,
                              "batch_step_ms": ms / steps,
                              "per_droplet_work_ms": {"p50": float(np.percentile(work, 50)),
                                                      "p99": float(np.percentile(work, 99)),
                                                      "basis": "share of the batch step by neighbour pairs"},
                              "dt_range": [float(rep["dt"].min()), float(rep["dt"].max())]}
        if rank == 0 and args.drop_long > 0 and prec == d.PREC_MIXED and (closure == d.CLOSURE_LEARNED or
                                                                            weights is None):
            long_form = name
            t0 = time.perf_counter()
            ctx.event_record(2)
            ctx.integrate_groups(args.drop_long, graph=True)
            ctx.event_record(3)
            ms_l = ctx.event_elapsed(2, 3)
            rep_l = ctx.group_report()
            out["long_run"] = {"form": name, "steps": args.drop_long, "value": total * args.drop_long / (ms_l / 1e3),
                               "unit": UNIT, "ms_per_step": ms_l / args.drop_long,
                               "wall_s": round(time.perf_counter() - t0, 1),
                               "sim_time_range_s": [float(rep_l["time"].min()), float(rep_l["time"].max())]}
        ctx.close()
    if rank == 0 and args.drop_sample > 0:
        order = np.argsort(full.counts)
        pick = order[np.linspace(0, len(order) - 1, min(args.drop_sample, len(order))).astype(int)]
        t_ms, ns = [], []
        for g in pick:
            c = full.single(int(g))
            s = c.settings.copy()
            s.precision = d.PREC_MIXED
            ctx = Context(s, c.state.n + 64, c.blocks)
            ctx.set_states(c.state, c.state)
            for _ in range(2):
                ctx.integrate()
            ctx.event_record(0)
            for _ in range(3):
                ctx.integrate()
            ctx.event_record(1)
            t_ms.append(ctx.event_elapsed(0, 1) / 3)
            ns.append(c.state.n)
            ctx.close()
        t_ms, ns = np.array(t_ms), np.array(ns, dtype=np.float64)
        a, b0 = np.polyfit(ns, t_ms, 1)
        seq_ms = float(np.sum(np.maximum(a * full.counts + b0, t_ms.min())))
        out["alone_fp32_plain_closure"] = {
            "sample": f"{len(pick)} droplets spread over the count range, one context each, 3 steps",
            "per_droplet_step_ms": {"p50": float(np.percentile(t_ms, 50)), "p99": float(np.percentile(t_ms, 99))},
            "sequential_step_ms_all_droplets": seq_ms,
            "value": total / (seq_ms / 1e3), "unit": UNIT}
    return out


def run_reference(args, threads: int, ws: int) -> dict:
    """The CPU restatement of the reference algorithm (the oracle) on the same workload: the live
    jet at the same cap, built with the oracle's own settings derivation (no GPU library is
    loaded), stepped with OpenMP on all host cores; each step counts the fluid particles it
    started with."""
    from fjsph_gb300 import cases
    from oracle import settings_ref
    from oracle.pyoracle import Oracle, set_threads
    cases.defaults, cases.derive = settings_ref.defaults, settings_ref.derive
    c = cases.jet_crossflow_live(n_target=args.n, cap=args.n)
    nb = c.state.n - c.n_fluid
    set_threads(threads)
    o = Oracle(c.settings, c.blocks, c.inlets)
    o.air_power_law(*c.power_law_params)
    o.set_states(c.state, c.state)
    for _ in range(min(args.warmup, 1)):
        o.integrate()
    ps = 0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ps += o.particle_count() - nb
        o.integrate()
    dt = time.perf_counter() - t0
    v = ps / dt
    sample = (f"the live-inlet jet itself ({c.state.n} particles at the start, cap {args.n}), "
              f"{args.steps} Integrator::integrate steps after {min(args.warmup, 1)} warm-up, OpenMP")
    return {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "particles": int(c.state.n), "fluid": int(c.n_fluid), "cap": args.n},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def side(fn, *a):
    """A side section of the line: its result, or {"error": ...} when it fails (the headline and
    the other sections are still reported)."""
    try:
        return fn(*a)
    except Exception as e:  # noqa: BLE001 -- reported in the line, not swallowed
        import traceback
        traceback.print_exc(file=sys.stderr)
        return {"error": f"{type(e).__name__}: {e}"}


def main():
    args = parse()
    ws, rank, local = dist_env()
    threads = os.cpu_count() or 1
    if args.impl == "reference":
        if rank != 0:
            return 0
        print(json.dumps(run_reference(args, threads, ws)))
        return 0
    if ws > 1:
        os.environ.setdefault("CUDA_VISIBLE_DEVICES", str(local))
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(0)
        dist.init_process_group("nccl")
    r = run_ours(args, ws, rank, local)
    drops = side(run_droplets, args, ws, rank, r["weights"]) if args.drops > 0 else None
    vlm = side(run_vlm, args) if (args.vlm_points > 0 and rank == 0) else None
    setup = side(run_case_setup, args) if (args.setup_particles > 0 and rank == 0) else None
    mesh = side(run_mesh, args, r["case"]) if (args.mesh_cell > 0 and rank == 0) else None
    cfg0 = side(run_config0, args, threads, rank) if (args.config0_steps > 0 and rank == 0) else None
    cfg1 = side(run_config1, args) if (args.config1_dx > 0 and rank == 0) else None
    if rank == 0:
        cpu = parity = None
        if not args.no_cpu:
            got = side(run_cpu_parity, args, r["case"], threads)
            cpu, parity = (got, got) if isinstance(got, dict) else got
        line = {"metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": r["ms"] / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None,
                "dtype": "f64" if args.precision == "fp64" else ("f32+f64+bf16" if args.closure == "learned" else "f32+f64"),
                "data": "synthetic",
                "config": {"workload": WORKLOAD, "particles": r["n"], "fluid": r["nf"], "cap": args.n,
                           "air": "50 m/s crossflow, 1/7-power-law boundary layer 5 mm over z = 0",
                           "form": args.precision, "closure": args.closure if args.precision == "mixed" else "plain",
                           "integrator": "runge_kutta4", "pairs": args.pairs,
                           "l2": "inputs larger than L2 (state ~1 GB)", "parallelism": f"replicas{ws}"},
                "roofline": r["roof"], "cpu_baseline": cpu, "e2e": r["e2e"], "clocks": r["clocks"],
                "parity": parity, "live_inlet": r["live"],
                "fp64_form": r["fp64"], "fp32_plain_closure_form": r["plain"],
                "speedup_vs_fp64_form": (r["value"] / r["fp64"]["value"]) if r["fp64"] else None,
                "closure": r["closure"], "neighbour_pairs": r["pairs"], "autotune": r["tune"],
                "residual_order": r["order"],
                "neighbour_pairs_per_s": r["pairs"] * args.steps * ws / (r["ms"] / 1e3),
                "gpu_launches": r["launches"], "passes_ms": r["prof"],
                "config0_dam_break_2d": cfg0, "config1_dam_break_3d": cfg1, "droplet_batch": drops,
                "vlm_air_source": vlm, "mesh_air_source": mesh, "case_setup": setup}
        print(json.dumps(line))
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
