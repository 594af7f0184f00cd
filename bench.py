"""Benchmark: Galerkin GEP assembly + sparse eigensolve on one GB300 (fem_2d's hot path).

Workload (default, `full_1m`): the full form at scale - [0,2]x[0,1] meshed as 64x32 base Elems,
per-Elem expansion orders uniform in 3..8 per direction, four seeded rounds of T/U/V h-refinement of
44% of the leaves (1,070,625 DoFs), HierPoly basis, GLQ [10,10]; the 20 eigenpairs nearest 10.0. A step
is one assembly (tables + values on the device) plus one gpu_solve_gep (two multifrontal
factorizations + the shift-invert block eigensolver).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl native|reference] [--workload NAME]

Prints one JSON line. `value` is DoFs/s with the GEP structures already resident in device memory;
`e2e` is the same metric through the public API from host data (host symbolic phase, uploads and the
eigenpair download inside the timed region; `e2e.phases` splits the last such step). Outside the timed
regions: `parity` (against the FP64 oracle: run here up to 60k DoFs, or read from the committed oracle
fixture of the workload, tests/golden/full_form_*.json, made by tests/golden/make_full_form_fixture.py)
and `accuracy` (the eigenvalues against the analytic eigenvalues of the PEC rectangle and against a solve
of the same mesh in the other basis). `cpu_baseline` times the oracle's CPU restatement of the path on
a bounded sample; the reference arm (`--impl reference`) times it on the workload itself, or prints an
`unavailable` line when the whole run would not fit the time limit.

Other workloads: `precision` (16x8 Elems, orders 6, KOLeg, 10 pairs, 28,818 DoFs), `full_160k`
(32x16 base Elems, 160,346 DoFs) and `batch` (256 seeded waveguide meshes: one batched assembly plus
256 concurrent solves per step).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "assembly+eigensolve s and DoFs/s, learned vs plain GPU, eig rel err<=1e-9"
UNIT = "DoFs/s"


# full-form workloads with a committed FP64 oracle fixture: name -> configs.full_scale arguments
FULL_FORM = {
    "full_1m": dict(nx=64, ny=32, rounds=4, fraction=0.44),
    "full_160k": dict(nx=32, ny=16, rounds=3, fraction=0.44),
}


def workload(name, replay=None):
    """The named workload; `replay` is the mesh class its refinement script is built on (the product's
    Mesh by default; the reference arm passes the oracle's, so it loads no product library)."""
    from fem_2d_gb300 import configs

    kw = {} if replay is None else {"replay": replay}
    if name == "precision":
        return configs.precision(seed=0, **kw)
    if name == "waveguide":
        return configs.waveguide_small(**kw)
    if name in FULL_FORM:
        return configs.full_scale(seed=0, basis=0, **FULL_FORM[name], **kw)
    if name == "full_small":
        return configs.full_scale(seed=0, nx=32, ny=16, rounds=3, **kw)
    if name == "full":
        return configs.full_scale(seed=0, **kw)
    if name == "full_koleg_1m":
        return configs.full_scale(seed=0, basis=1, fraction=0.44, **kw)
    raise SystemExit("unknown workload " + name)


def fixture(name):
    """The committed FP64 oracle fixture of a full-form workload, or None."""
    p = os.path.join(ROOT, "tests", "golden", "full_form_%s.json" % name)
    if name not in FULL_FORM or not os.path.exists(p):
        return None
    with open(p) as f:
        return json.load(f)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def barrier_max(value, ws):
    """max over ranks (host float); plain pass-through for one process"""
    if ws == 1:
        return value
    import torch
    import torch.distributed as dist

    t = torch.tensor([value], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = tempfile.mktemp(prefix="fem2d_clocks_", suffix=".csv")

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                p = [x.strip() for x in line.split(",")]
                if len(p) < 9:
                    continue
                try:
                    sm.append(float(p[1]))
                    mx.append(float(p[2]))
                except ValueError:
                    continue
                for k, nm in enumerate(names):
                    if p[5 + k].lower().startswith("active"):
                        reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def profile_traffic():
    """DRAM bytes per launch of the dominant kernel from the committed ncu summary, if present."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return {}


def oracle_check(w, key, gep, res):
    """Parity against the FP64 oracle, outside every timed region. Up to 60k DoFs the oracle runs here
    (literal assembly + FP64 sparse shift-invert); a full-form workload with a committed oracle fixture
    is checked against it (pattern hash bit for bit, a seeded sample of entries, the 20 eigenvalues)."""
    import hashlib

    import numpy as np

    fx = fixture(key)
    if fx is not None:
        gr, gc, ga, gb = gep.upper_coo()
        h = hashlib.sha256()
        h.update(np.ascontiguousarray(gr, dtype="<i4").tobytes())
        h.update(np.ascontiguousarray(gc, dtype="<i4").tobytes())
        sm = fx["sample"]
        key_g = gr.astype(np.int64) * gep.dimension + gc
        key_s = np.asarray(sm["rows"], np.int64) * gep.dimension + np.asarray(sm["cols"], np.int64)
        pos = np.searchsorted(key_g, key_s)
        pos = np.minimum(pos, len(key_g) - 1)
        found = bool(np.all(key_g[pos] == key_s))
        ea = float(np.max(np.abs(ga[pos] - np.asarray(sm["a"]))) / fx["max_abs_a"])
        eb = float(np.max(np.abs(gb[pos] - np.asarray(sm["b"]))) / fx["max_abs_b"])
        del gr, gc, ga, gb, key_g
        ov = np.asarray(fx["eigenvalues"])
        gv = np.sort(res.values)
        m = min(len(ov), len(gv))
        # each oracle eigenvalue against the nearest GPU eigenvalue (equal counts when both found all pairs)
        rel = np.array([np.min(np.abs(gv - t)) / abs(t) for t in ov[:m]])
        out = {"oracle": "committed FP64 oracle fixture (tests/golden/full_form_%s.json): literal 2-D assembly + "
                         "ARPACK shift-invert Lanczos with SuperLU solves; eigenvalues from the %s pencil"
                         % (key, fx.get("eig_pencil", "HierPoly").split(" ")[0]),
               "ndofs_match": gep.dimension == fx["ndofs"], "nnz_upper_match": gep.dims()[1] == fx["nnz_upper"],
               "pattern_bit_exact": h.hexdigest() == fx["pattern_sha256"], "sample_keys_found": found,
               "sample_entries": len(key_s), "entry_err_A": ea, "entry_err_B": eb,
               "eig_rel_err_max": float(np.max(rel)), "eig_rel_err": rel.tolist(), "pairs_compared": int(m),
               "oracle_rr_vs_mu_max_rel_diff": fx.get("rr_vs_mu_max_rel_diff"),
               "oracle_err_bound_rel_max": (float(np.max(np.asarray(fx["rr_err_bound"]) / np.abs(np.asarray(fx["rr_eigenvalues"]))))
                                            if fx.get("rr_err_bound") else None)}
        if "cross_check" in fx:
            out["oracle_methods_max_rel_diff"] = fx["cross_check"]["max_rel_diff"]
        return out
    if gep.dimension > 60000:
        return {"skipped": "no oracle fixture for this workload; the oracle's solve runs here only up to 60k DoFs"}
    from oracle import ref

    om = ref.OracleMesh(w.mesh_json)
    om.apply_ops(w.ops)
    n = om.domain()
    r, c, a, b = om.galerkin(w.basis, w.glq[0], w.glq[1], threads=os.cpu_count() or 4)
    gr, gc, ga, gb = gep.upper_coo()
    same = bool(np.array_equal(r, gr) and np.array_equal(c, gc))
    ea = float(np.max(np.abs(ga - a)) / np.max(np.abs(a)))
    eb = float(np.max(np.abs(gb - b)) / np.max(np.abs(b)))
    A = ref.full_sym(n, r, c, a)
    B = ref.full_sym(n, r, c, b)
    perm = ref.nd_order(ref.dof_boxes(om))
    ws = ref.arpack_nearest_physical(A, B, w.target, w.n_pairs, perm, refine=0)["values"]
    rel = float(np.max(np.abs(np.sort(res.values) - np.sort(ws)) / np.abs(np.sort(ws))))
    return {"oracle": "FP64 oracle run here: literal 2-D assembly + ARPACK shift-invert Lanczos with SuperLU solves",
            "pattern_bit_exact": same, "entry_err_A": ea, "entry_err_B": eb, "eig_rel_err_max": rel}


def cpu_port_step(w, threads):
    """One step of the CPU restatement of the path (the oracle, on the host cores): the literal 2-D
    quadrature assembly on `threads` threads, then the FP64 sparse shift-invert eigensolve (ARPACK
    Lanczos on T with SuperLU solves under the oracle's nested-dissection ordering). Returns
    (ndofs, assembly s, eigensolve s)."""
    from oracle import ref

    t0 = time.perf_counter()
    om = ref.OracleMesh(w.mesh_json)
    om.apply_ops(w.ops)
    n = om.domain()
    r, c, a, b = om.galerkin(w.basis, w.glq[0], w.glq[1], threads=threads)
    t1 = time.perf_counter()
    A = ref.full_sym(n, r, c, a)
    B = ref.full_sym(n, r, c, b)
    perm = ref.nd_order(ref.dof_boxes(om))
    ref.arpack_nearest_physical(A, B, w.target, w.n_pairs, perm, refine=0)
    t2 = time.perf_counter()
    return n, t1 - t0, t2 - t1


# the bounded CPU sample of a full-form workload: the family's 16x8-base-Elem member (same orders,
# rounds and refinement fraction), one full step of the CPU port
def cpu_sample(name, replay=None):
    from fem_2d_gb300 import configs

    if name in FULL_FORM:
        kw = dict(FULL_FORM[name], nx=16, ny=8)
        if replay is not None:
            kw["replay"] = replay
        return configs.full_scale(seed=0, basis=0, **kw), "the full-form family's 16x8-base-Elem member"
    return workload(name, replay), "the workload itself"


def reference_config(w, n):
    return {"workload": w.name, "ndofs": n, "basis": "KOLeg" if w.basis == 1 else "HierPoly", "glq": list(w.glq),
            "n_pairs": w.n_pairs, "target": w.target, "seed": w.seed}


def run_reference(args, ws, rank):
    """The reference arm: the oracle's CPU restatement of the reference's path (literal 2-D quadrature
    assembly on all host threads + FP64 sparse shift-invert eigensolve) on the same workload. Workload
    scripts are replayed on the oracle's mesh, so no product library is loaded. When the committed
    fixture's single-step time says that W + K steps cannot finish within the run limit, an
    `unavailable` line says so instead."""
    if rank != 0:
        return
    from oracle import build as ob

    ob.build_oracle()
    from oracle import ref

    w = workload(args.workload, ref.OracleReplay)
    threads = os.cpu_count() or 4
    fx = fixture(args.workload)
    if fx is not None:
        one = fx["t_oracle_assembly_s"] + fx["t_oracle_eigensolve_s"]
        if one * (args.steps + args.warmup) > args.reference_limit_s:
            print(json.dumps({
                "impl": "reference", "metric": METRIC, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "higher_is_better": True,
                "config": dict(reference_config(w, fx["ndofs"]), nnz_upper=fx["nnz_upper"]),
                "unavailable": "one step of the CPU restatement of the path at %d DoFs takes at least %.0f s on %d host "
                               "threads (literal assembly %.0f s + FP64 ARPACK shift-invert with substructured SuperLU "
                               "solves %.0f s on the %s pencil); %d steps would take about %.0f s, beyond the %d s limit; "
                               "the native line's cpu_baseline times a bounded sample"
                               % (fx["ndofs"], one, fx["threads"], fx["t_oracle_assembly_s"], fx["t_oracle_eigensolve_s"],
                                  fx.get("eig_pencil", "HierPoly").split(" ")[0], args.steps + args.warmup,
                                  one * (args.steps + args.warmup), args.reference_limit_s)}), flush=True)
            return
    for _ in range(args.warmup):
        cpu_port_step(w, threads)
    tot, ta, te, n = 0.0, 0.0, 0.0, 0
    for _ in range(args.steps):
        n, a, e = cpu_port_step(w, threads)
        tot += a + e
        ta += a
        te += e
    v = n * args.steps / tot
    out = {"metric": METRIC, "value": v, "unit": UNIT, "impl": "reference", "n_gpus": ws, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1e3 * tot / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded mesh family)",
           "config": reference_config(w, n),
           "t_assembly_s": ta / args.steps, "t_eigensolve_s": te / args.steps,
           "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                            "sample": "full workload per step: literal 2-D quadrature assembly on %d threads + FP64 sparse "
                                      "shift-invert (ARPACK Lanczos, SuperLU under nested dissection)" % threads},
           "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def learned_vs_plain(ctx, eval_nx=16, eval_ny=8, train_nx=8, train_ny=4, shift=10.0, k=4, hidden=64,
                     epochs=300, n_pairs=10):
    """The metric's learned-vs-plain comparison on the learned-preconditioner family (KOLeg, orders (5,7),
    two rounds of U/V refinement): gpu_solve_gep for the 10 pairs nearest 10.0 with iterative inner solves
    (CG on A + 10 B, MINRES on A - 10 B), once with the plain additive-Schwarz preconditioner and once
    with the learned two-level preconditioner, on the held-out seed 4 at eval_nx x eval_ny base Elems
    (16 x 8 by default, 34,570 DoFs, about two minutes for both arms; `--learned-full` runs the family's
    full 32 x 16 size, 138,861 DoFs);
    both to the same outer tolerance, each timed end to end (preconditioner set-up included) and checked
    against the exact multifrontal path's eigenvalues. The per-Elem-patch network is trained on the GPU
    by the library's own kernels on error vectors of the plain solver (harvest_errors) on seeds 1..3 at
    train_nx x train_ny."""
    import numpy as np

    import fem_2d_gb300 as fg
    from fem_2d_gb300 import configs

    def gep(seed, nx, ny):
        w = configs.learned_family(seed, nx, ny)
        d = fg.Domain.from_mesh(configs.build_mesh(w))
        return d, fg.galerkin_sample_gep_hcurl(fg.KOLeg, fg.CurlCurl, fg.L2Inner, d, [10, 10], ctx=ctx)

    t0 = time.perf_counter()
    train = [gep(s, train_nx, train_ny) for s in (1, 2, 3)]
    samples = []
    for _, gt in train:
        E = fg.harvest_errors(gt, 1.0, shift, nrhs=16, every=2, max_samples=256, seed=1, first=100)
        samples.append(np.vstack([E] * (256 // max(1, len(E)) + 1))[:256])
    t1 = time.perf_counter()
    net = fg.PatchNet(k=k, hidden=hidden, seed=0)
    hist = net.train([gt for _, gt in train], shift, samples, epochs=epochs, lr=2e-3)
    t2 = time.perf_counter()
    npatch = sum(len(fg.patch_features(d, shift)[0]) - 1 for d, _ in train)
    d, g = gep(4, eval_nx, eval_ny)
    exact = fg.gpu_solve_gep_n(g, shift, n_pairs)
    ev = np.sort(exact.values)
    out = {"workload": "learned_%dx%d_p5-7_koleg_seed4_heldout" % (eval_nx, eval_ny), "ndofs": g.dimension,
           "n_pairs": n_pairs, "target": shift,
           "inner": "CG on A + 10 B and MINRES on A - 10 B to 1e-10 relative residual per inner solve",
           "train": {"meshes": "learned_%dx%d seeds 1..3" % (train_nx, train_ny), "error_vectors": 3 * 256,
                     "patch_samples": 256 * npatch, "params": net.num_params, "coarse_vectors_per_elem": k,
                     "harvest_s": t1 - t0, "train_s": t2 - t1,
                     "loss_first_last": [float(hist[0]), float(hist[-1])]},
           "exact_multifrontal_s": exact.stats["t_setup_ms"] / 1e3 + exact.stats["t_solve_ms"] / 1e3}
    for name, pc, nn in (("plain", fg.PRECOND_PLAIN, None), ("learned", fg.PRECOND_LEARNED, net)):
        ctx.synchronize()
        ts = time.perf_counter()
        r = fg.gpu_solve_gep_n(g, shift, n_pairs, precond=pc, net=nn)
        te = time.perf_counter() - ts
        out[name] = {"s": te, "outer_cycles": r.stats["outer_iters"], "cg_iters": r.stats["inner_cg_iters"],
                     "minres_iters": r.stats["inner_minres_iters"], "setup_ms": r.stats["t_setup_ms"],
                     "max_rel_residual": float(np.max(r.residuals)),
                     "eig_rel_err_vs_exact": float(np.max(np.abs(np.sort(r.values) - ev) / np.abs(ev)))}
    out["speedup_learned_over_plain"] = out["plain"]["s"] / out["learned"]["s"]
    out["target_speedup"] = 3.0
    return out


def run_native(args, ws, rank, local):
    import numpy as np

    import fem_2d_gb300 as fg
    from fem_2d_gb300 import configs

    w = workload(args.workload)
    bs = fg.KOLeg if w.basis == 1 else fg.HierPoly
    ctx = fg.Context(local)
    mesh = configs.build_mesh(w)
    dom = fg.Domain.from_mesh(mesh)
    n = dom.num_dofs
    gep = fg.galerkin_sample_gep_hcurl(bs, fg.CurlCurl, fg.L2Inner, dom, list(w.glq), ctx=ctx)
    _, nnz_u, nnz_f = gep.dims()

    def step():
        ctx.timer_start()
        gep.recompute()
        ta = ctx.timer_stop()
        ctx.timer_start()
        res = fg.gpu_solve_gep_n(gep, w.target, w.n_pairs, dense=args.dense, refine=args.refine,
                                 krylov_steps=args.krylov_steps, block=args.block)
        te = ctx.timer_stop()
        return ta, te, res

    for _ in range(args.warmup):
        step()
    ctx.synchronize()
    barrier(ws)
    sampler = ClockSampler(local) if rank == 0 else None
    if sampler:
        sampler.start()
    l0 = ctx.kernel_launches
    t_asm = t_eig = 0.0
    res = None
    wall0 = time.perf_counter()
    for _ in range(args.steps):
        ctx.flush_l2()
        ctx.synchronize()
        ta, te, res = step()
        t_asm += ta
        t_eig += te
    ctx.synchronize()
    wall = time.perf_counter() - wall0
    launches = ctx.kernel_launches - l0
    clocks = sampler.stop() if sampler else None
    barrier(ws)
    ms_step = barrier_max((t_asm + t_eig) / args.steps, ws)
    value = ws * n / (ms_step / 1e3)

    # end to end through the public API from host data (at most 5 repetitions: at 1M DoFs one takes ~6 s)
    e2e_ms = 0.0
    h2d = d2h = 0
    parts = {}
    e2e_reps = max(1, min(args.steps, 5))
    for _ in range(e2e_reps):
        ctx.synchronize()
        t0 = time.perf_counter()
        d2 = fg.Domain.from_mesh(mesh)
        t1 = time.perf_counter()
        g2 = fg.galerkin_sample_gep_hcurl(bs, fg.CurlCurl, fg.L2Inner, d2, list(w.glq), ctx=ctx)
        t2 = time.perf_counter()
        r2 = fg.gpu_solve_gep_n(g2, w.target, w.n_pairs, dense=args.dense, refine=args.refine,
                                krylov_steps=args.krylov_steps, block=args.block)
        t3 = time.perf_counter()
        e2e_ms += 1e3 * (t3 - t0)
        tg = g2.timings()
        # the last iteration's phases (ms): host DoF enumeration, GEP construction (host symbolic
        # phase, uploads, device assembly), solve set-up (factorization plan, scaling, factorizations)
        # and Krylov phase, download included in the solve
        parts = {"domain_ms": 1e3 * (t1 - t0), "gep_ms": 1e3 * (t2 - t1), "gep_symbolic_ms": float(tg[3]),
                 "gep_upload_ms": float(tg[4]), "gep_assembly_ms": float(tg[2]), "solve_ms": 1e3 * (t3 - t2),
                 "solve_setup_ms": r2.stats["t_setup_ms"], "solve_krylov_ms": r2.stats["t_solve_ms"]}
        h2d = g2.h2d_bytes + 8 * n * (w.n_pairs + max(4, w.n_pairs // 2))
        d2h = 8 * w.n_pairs * (n + 2)
        del g2, d2, r2
    e2e_ms = barrier_max(e2e_ms / e2e_reps, ws)
    e2e = ws * n / (e2e_ms / 1e3)

    # profiling pass (one extra step, per-region CUDA events) for the roofline
    ctx.profile_reset()
    ctx.set_profiling(True)
    ctx.synchronize()
    tp0 = time.perf_counter()
    step()
    ctx.synchronize()
    ms_prof = 1e3 * (time.perf_counter() - tp0)
    ctx.set_profiling(False)
    regions = {}
    for reg in ("assembly_values", "spmm", "spmm_tc", "spmm_slice", "mf_factor", "mf_solve", "dense_block", "gram_tc",
                "gemm_tc", "vector_ops", "block_scale", "rr_host"):
        regions[reg] = ctx.profile(reg)
    dom_name = max(regions, key=lambda k: regions[k]["ms"])
    hbm, peak_kind = peaks()
    fp64 = ctx.fp64_peak()
    # issue cost of one tcgen05.mma (M = 128, K = 16) by N: the cost model of the tensor-core kernels
    mma_ns = {str(nn): round(ctx.mma_ns(nn), 2) for nn in (32, 64, 128, 256)}

    def roof(reg):
        """The region's achieved HBM bandwidth and FP64 rate against the measured peaks; `bound` is the
        resource the region uses the larger fraction of (GB300's FP64 rate bounds the multi-column
        operator products and the front products before HBM does)."""
        r = regions[reg]
        if r["count"] == 0 or r["ms"] <= 0:
            return None
        gbs = r["bytes"] / (r["ms"] / 1e3) / 1e9
        tfl = r["flops"] / (r["ms"] / 1e3) / 1e12
        f_hbm, f_fp = gbs / hbm, tfl / fp64
        base = {"launches": r["count"], "avg_launch_ms": r["ms"] / r["count"],
                "alg_bytes_per_launch": r["bytes"] / r["count"], "alg_flops_per_launch": r["flops"] / r["count"],
                "hbm": {"achieved": gbs, "peak": hbm, "unit": "GB/s", "frac": f_hbm, "peak_source": peak_kind},
                "fp64": {"achieved": tfl, "peak": fp64, "unit": "TFLOP/s", "frac": f_fp,
                         "peak_source": "measured (library FP64 FMA microbenchmark, this run)"}}
        if reg == "rr_host":
            # dense Rayleigh-Ritz on the host CPU: its FLOP rate is reported, no device roofline applies
            base.update({"bound": "host", "achieved": tfl, "peak": None, "unit": "TFLOP/s", "frac": None,
                         "note": "host CPU work (symmetric eigen-decompositions and products of the basis size)"})
            base["fp64"]["frac"] = None
            base["hbm"]["frac"] = None
            return base
        if reg in ("gram_tc", "gemm_tc", "spmm_tc"):
            # FP64 emulated on the tensor cores: its FP64-equivalent rate is not bounded by the FP64 pipe;
            # the kernel streams its operands once, so HBM is its roofline (tensor-pipe use from ncu)
            base["fp64"]["note"] = "FP64-equivalent rate of the tensor-core emulation (may exceed the FP64 peak)"
            base.update({"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s", "frac": f_hbm})
        elif f_fp > f_hbm:
            base.update({"bound": "fp64", "achieved": tfl, "peak": fp64, "unit": "TFLOP/s", "frac": f_fp})
        else:
            base.update({"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s", "frac": f_hbm})
        return base

    roofline = roof(dom_name)
    traffic = profile_traffic().get(w.name, {}).get(dom_name)
    roofline["kernel"] = dom_name
    roofline["traffic"] = traffic
    share = {k: regions[k]["ms"] for k in regions}

    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded mesh family)",
           "config": {"workload": w.name, "ndofs": n, "nnz_upper": nnz_u, "nnz_full": nnz_f,
                      "visits": gep.num_visits, "basis": "KOLeg" if w.basis == 1 else "HierPoly",
                      "glq": list(w.glq), "n_pairs": w.n_pairs, "target": w.target, "seed": w.seed,
                      "precond": "exact multifrontal shift-invert solves (the eigensolve with iterative inner "
                                 "solves, plain vs learned preconditioner, is measured in learned_vs_plain)",
                      "l2": "256 MiB device write between timed steps", "parallelism": "replicas" if ws > 1 else "1 GPU"},
           "t_assembly_s": t_asm / args.steps / 1e3, "t_eigensolve_s": t_eig / args.steps / 1e3,
           "wall_s_timed": wall, "gpu_launches": launches,
           "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                   "ms_per_step": e2e_ms, "steps": e2e_reps, "phases": parts},
           "roofline": roofline, "region_ms_profiled": share,
           "region_ms_unprofiled": ms_prof - sum(share.values()), "ms_profiled_step": ms_prof,
           "region_rooflines": {k: roof(k) for k in regions if k != dom_name},
           "solve_stats": res.stats if res is not None else None,
           "max_rel_residual": float(np.max(res.residuals)) if res is not None else None,
           "clocks": clocks, "tensor_mma_ns_per_sm": mma_ns}
    if rank == 0 and not args.no_check:
        out["parity"] = oracle_check(w, args.workload, gep, res)
    if rank == 0 and not args.no_check:
        out["accuracy"] = accuracy_check(w, mesh, ctx, res)
    if rank == 0 and ws == 1 and not args.no_learned:
        out["learned_vs_plain"] = (learned_vs_plain(ctx, 32, 16, 16, 8) if args.learned_full else learned_vs_plain(ctx))
    if rank == 0 and ws == 1 and not args.no_cpu:
        threads = os.cpu_count() or 4
        sw, what = cpu_sample(args.workload)
        cn, ca_, ce = cpu_port_step(sw, threads)
        out["cpu_baseline"] = {"value": cn / (ca_ + ce), "unit": UNIT, "cores": threads, "kind": "port",
                               "sample": "one full step of %s (%s, %d DoFs): literal 2-D quadrature assembly "
                                         "(%.2f s) + FP64 ARPACK/SuperLU shift-invert (%.2f s)"
                                         % (what, sw.name, cn, ca_, ce)}
    if rank == 0:
        print(json.dumps(out), flush=True)


def accuracy_check(w, mesh, ctx, res):
    """Size-independent eigenvalue checks, outside every timed region. The meshes cover [0,2]x[0,1] with
    PEC walls, whose Maxwell eigenvalues are (m pi / 2)^2 + (k pi)^2; and HierPoly and KOLeg span the
    same discrete space on a mesh, so the other basis gives the same Galerkin eigenvalues up to rounding
    (a second, independently assembled and solved pencil)."""
    import numpy as np

    import fem_2d_gb300 as fg

    vals = np.sort(res.values)
    ana = np.sort([(a * np.pi / 2) ** 2 + (b * np.pi) ** 2 for a in range(0, 40) for b in range(0, 20) if a + b > 0])
    near = np.sort(ana[np.argsort(np.abs(ana - w.target), kind="stable")[: len(vals)]])
    other = fg.HierPoly if w.basis == 1 else fg.KOLeg
    dom = fg.Domain.from_mesh(mesh)
    g2 = fg.galerkin_sample_gep_hcurl(other, fg.CurlCurl, fg.L2Inner, dom, list(w.glq), ctx=ctx)
    t0 = time.perf_counter()
    r2 = fg.gpu_solve_gep_n(g2, w.target, w.n_pairs)
    t2 = time.perf_counter() - t0
    v2 = np.sort(r2.values)
    return {"max_rel_err_vs_analytic_waveguide": float(np.max(np.abs(vals - near) / near)),
            "other_basis": "HierPoly" if w.basis == 1 else "KOLeg",
            "max_rel_diff_vs_other_basis": float(np.max(np.abs(vals - v2) / np.abs(v2))),
            "other_basis_solve_s": t2, "other_basis_stats": r2.stats,
            "backward_error": res.stats.get("max_backward_error")}


def run_native_batch(args, ws, rank, local):
    """The batching family: 256 independent seeded meshes; all element integrals of all meshes in one
    table launch plus one persistent autotuned value launch, then the 4 pairs nearest 10.0 of every
    mesh by concurrent per-mesh solves (one CUDA stream per worker thread). A step is one batched
    assembly plus all 256 solves; it spans several streams, so it is timed on the host around a
    device-wide synchronisation on both sides."""
    import numpy as np

    import fem_2d_gb300 as fg
    from fem_2d_gb300 import configs

    count = args.batch_count
    wl = [configs.batch_member(s) for s in range(count)]
    ctx = fg.Context(local)
    doms = [fg.Domain.from_mesh(configs.build_mesh(w)) for w in wl]
    ndofs = sum(d.num_dofs for d in doms)
    t0 = time.perf_counter()
    geps, rep = fg.galerkin_sample_gep_hcurl_batch(fg.HierPoly, fg.CurlCurl, fg.L2Inner, doms, [10, 10], ctx=ctx)
    t_first = time.perf_counter() - t0
    workers = args.workers

    def step():
        r = fg.gep_batch_recompute(geps, ctx=ctx)
        ctx.synchronize()
        ta = time.perf_counter()
        res = fg.gpu_solve_gep_batch(geps, 10.0, 4, workers=workers, dense=args.dense, refine=args.refine)
        return r, res, ta

    for _ in range(args.warmup):
        step()
    barrier(ws)
    sampler = ClockSampler(local) if rank == 0 else None
    if sampler:
        sampler.start()
    l0 = ctx.kernel_launches
    tot = t_asm_dev = t_solve = 0.0
    res = None
    for _ in range(args.steps):
        ctx.flush_l2()
        ctx.synchronize()
        t0 = time.perf_counter()
        r, res, ta = step()
        t1 = time.perf_counter()
        tot += t1 - t0
        t_solve += t1 - ta
        t_asm_dev += r["ms_tables"] + r["ms_values"]
    clocks = sampler.stop() if sampler else None
    ms_step = barrier_max(1e3 * tot / args.steps, ws)
    value = ws * ndofs / (ms_step / 1e3)
    worst = max(float(np.max(x.residuals)) for x in res)
    hbm, peak_kind = peaks()
    r = fg.gep_batch_recompute(geps, ctx=ctx)
    # A and B written (16 B per entry), the upper entry each entry mirrors (4 B), the visit ranges of the
    # upper entries (8 B each, plus one per GEP) and the visit codes (8 B each)
    upper = sum(g.dims()[1] for g in geps)
    alg = 20.0 * r["entries"] + 8.0 * (upper + len(geps)) + 8.0 * r["codes"]
    achieved = alg / (r["ms_values"] / 1e3) / 1e9
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (seeded mesh family)",
           "config": {"workload": "batch_%d_waveguides_p2-8_hierpoly" % count, "meshes": count, "ndofs_total": ndofs,
                      "ndofs_min": min(d.num_dofs for d in doms), "ndofs_max": max(d.num_dofs for d in doms),
                      "glq": [10, 10], "n_pairs": 4, "target": 10.0, "solve_workers": workers,
                      "timing": "host clock around device-wide sync (step spans %d streams)" % (workers + 1),
                      "l2": "256 MiB device write between timed steps",
                      "parallelism": "replicas" if ws > 1 else "1 GPU"},
           "t_assembly_device_s": t_asm_dev / args.steps / 1e3, "t_solves_s": t_solve / args.steps,
           "t_first_batch_with_symbolic_s": t_first,
           "gpu_launches": ctx.kernel_launches - l0,
           "assembly_launch": {"threads": r["threads"], "ctas_per_sm": r["ctas_per_sm"], "entries": r["entries"],
                               "ms_tables": r["ms_tables"], "ms_values": r["ms_values"]},
           "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                        "kernel": "fem2d_values_batch_kernel", "alg_bytes_per_launch": alg, "peak_source": peak_kind,
                        "traffic": None},
           "max_rel_residual": worst, "clocks": clocks}
    if rank == 0:
        print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    ap.add_argument("--workload", default="full_1m")
    ap.add_argument("--reference-limit-s", type=int, default=1500)
    ap.add_argument("--dense", type=int, default=0,
                    help="the eigensolver's contraction mode (fem2d_solve_opts.dense): 0 default, 1 FP64 CUDA "
                         "cores, 2 tensor-core operator products at every size, 3 FP64 operator products")
    ap.add_argument("--refine", type=int, default=0,
                    help="FP64 refinement steps per exact shifted solve (fem2d_solve_opts.refine): 0 calibrated "
                         "(default), k > 0 fixed, -1 none")
    ap.add_argument("--krylov-steps", type=int, default=0,
                    help="block Krylov steps per restart cycle (fem2d_solve_opts.krylov_steps), 0 = default")
    ap.add_argument("--block", type=int, default=0, help="eigensolver block size (fem2d_solve_opts.block), 0 = default")
    ap.add_argument("--no-check", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-learned", action="store_true")
    ap.add_argument("--learned-full", action="store_true")
    ap.add_argument("--batch-count", type=int, default=256)
    ap.add_argument("--workers", type=int, default=8)
    args = ap.parse_args()
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
    if args.impl == "reference":
        run_reference(args, ws, rank)
    elif args.workload == "batch":
        run_native_batch(args, ws, rank, local)
    else:
        run_native(args, ws, rank, local)
    if ws > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
