#!/usr/bin/env python3
"""Paillier-2048 throughput on one GB300 (HEU paillier_z semantics).

Workload (one step): one 2048-bit key (seed 0); 1,048,576 int64 plaintexts
m ~ U[-2^40, 2^40) with injected 1024-bit r; Encrypt (fixed-base h_s^r),
ciphertext Add (ct + ct'), scalar Mul by 64-bit k ~ U[-2^63, 2^63), CRT
Decrypt of the sums.  value = 4 * 2^20 ops per step / step time, with every
input already resident in HBM (512 MiB of ciphertexts per array, larger than
the 129 MB L2, so no flush is needed between steps).  e2e repeats the step
through the host-pointer C-ABI (hg_encrypt / hg_add / hg_mul / hg_decrypt)
with pinned host buffers, so every copy is inside the timed region.

--impl reference times the paillier_z CPU path (the oracle's C restatement;
HEU itself needs Bazel + yacl and does not build here) on all host cores,
each step a bounded sample of the same workload.
"""

import argparse
import ctypes
import json
import os

# before any CUDA context exists: every stream its own hardware work queue
# (the request server's slots must not queue behind one another's kernels)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

KEY_BITS = 2048
KEY_SEED = 0
M_BITS = 40
METRIC = "Paillier-2048 ops/s (enc/dec/mul/sum) and serve p99 ms, batched vs plain GPU"
UNIT = "ops/s"
WORKLOAD = "config2: 2048-bit key, 2^20 int64 m~U[-2^40,2^40), enc+add+mul(64-bit k)+CRT dec per step"


def mm_macs(limbs):
    """Montgomery multiplication cost in 32x32 MACs: 2s^2 + s."""
    return 2 * limbs * limbs + limbs


def decrypt_macs(key_bits, wd=6):
    """Algorithmic MACs of one CRT decryption (two (k/2)-bit exponentiations
    mod p^2, q^2 with sliding windows of wd bits, plus 3 MM for L and CRT)."""
    h = key_bits // 2
    sp = key_bits // 32
    steps = (h - 1) + -(-h // (wd + 1)) + 2 ** (wd - 1)
    return 2 * steps * mm_macs(sp) + 3 * mm_macs(sp)


def encrypt_macs(key_bits, w):
    return (-(-(key_bits // 2) // w) + 2) * mm_macs(key_bits // 16)


def mul_macs(key_bits, ks, wm=4):
    tot = 0
    for k in ks:
        b = abs(int(k)).bit_length()
        if b == 0:
            continue
        tot += (b - 1 + -(-b // (wm + 1)) + 2 ** (wm - 1) + 2)
    return tot * mm_macs(key_bits // 16)


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.out = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.out, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.out.close()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ---------------------------------------------------------------------------
def cpu_sample(seconds_hint=10.0, threads=None):
    """Time the paillier_z C restatement on a bounded sample of the workload.

    Returns per-op rates (ops/s) and the step-equivalent rate for the
    enc+add+mul+dec mix."""
    import numpy as np

    from oracle import cref
    from oracle import paillier_z as pz

    threads = threads or os.cpu_count() or 1
    pk, sk = pz.keygen(KEY_BITS, KEY_SEED)
    ck = cref.CKey(KEY_BITS, pk, sk, window=10)
    rng = np.random.default_rng(7)
    n_fast = 512 * threads
    n_dec = 96 * threads
    m = rng.integers(-(2 ** M_BITS), 2 ** M_BITS, size=n_fast, dtype=np.int64)
    r = rng.integers(0, 2 ** 63, size=(n_fast, ck.r_limbs), dtype=np.int64).astype(np.uint64) * 2 + 1
    k = rng.integers(-(2 ** 63), 2 ** 63 - 1, size=n_fast, dtype=np.int64)
    rates = {}
    t = time.perf_counter()
    ct = ck.encrypt(m, r, threads)
    rates["encrypt"] = n_fast / (time.perf_counter() - t)
    t = time.perf_counter()
    cs = ck.add(ct, ct[::-1].copy(), threads)
    rates["add"] = n_fast / (time.perf_counter() - t)
    n_mul = 128 * threads
    t = time.perf_counter()
    ck.mul(ct[:n_mul].copy(), k[:n_mul], threads)
    rates["mul"] = n_mul / (time.perf_counter() - t)
    t = time.perf_counter()
    d, _ = ck.decrypt(cs[:n_dec].copy(), threads)
    rates["decrypt"] = n_dec / (time.perf_counter() - t)
    assert np.array_equal(d, (m + m[::-1])[:n_dec]), "CPU baseline decrypt mismatch"
    step_rate = 4.0 / sum(1.0 / rates[o] for o in ("encrypt", "add", "mul", "decrypt"))
    # reductions (numpy/evaluator.cc:208-458) on the same ciphertexts
    ctc = np.ascontiguousarray(ct)
    t = time.perf_counter()
    for _ in range(4):
        ck.sum_mt(ctc, threads)
    rates["sum"] = 4 * n_fast / (time.perf_counter() - t)
    nb_rows, F, B = min(n_fast, 4096), 64, 256
    om = rng.integers(0, B, size=(nb_rows, F)).astype(np.uint8)
    t = time.perf_counter()
    ck.bucket_sum(ctc[:nb_rows], om, B, threads)
    rates["bucket_sum_row_features"] = nb_rows * F / (time.perf_counter() - t)
    Mm, K, N = 1, 256, 32
    y = rng.integers(-(2 ** 15), 2 ** 15, size=(K, N), dtype=np.int64)
    t = time.perf_counter()
    ck.matmul(ctc[: Mm * K].reshape(Mm, K, -1), y, threads)
    rates["matmul_outputs"] = Mm * N / (time.perf_counter() - t)
    sample = (f"{n_fast} encrypt+add, {n_mul} mul (64-bit k), {n_dec} CRT decrypt on 2048-bit key; "
              "step-equivalent rate = 4/(sum 1/rate_op); reductions: Sum of {0} x4, bucket-sum {1} rows x 64 "
              "features x 256 buckets, MatMul {2}x256 @ 256x32 int32 (per-element Mul + reduce as "
              "numpy/evaluator.cc)".format(n_fast, nb_rows, Mm))
    return rates, step_rate, threads, sample


def parity_sample(kp, m, r, kk, ct, cm, cs, ct2, count=4096):
    """Checker only, after the timed region: a strided sample of the timed
    outputs (Encrypt at the bench's table window, Add, Mul by 64-bit k)
    compared byte for byte, in Montgomery form, with the paillier_z C
    restatement given the same m, r and k.  Returns the number of
    ciphertexts compared; raises on any mismatch."""
    import numpy as np

    from oracle import cref
    from oracle import paillier_z as pz

    n = ct.shape[0]
    step = max(1, n // count)
    idx = np.arange(0, n, step)[:count]
    # include the last element as well (strided samples may miss the tail)
    idx[-1] = n - 1
    pk, sk = pz.keygen(KEY_BITS, KEY_SEED)
    assert pk.n == kp["n"], "bench key differs from the oracle key"
    ck = cref.CKey(KEY_BITS, pk, sk, window=10)
    threads = os.cpu_count() or 1
    ti = __import__("torch").from_numpy(idx).to(ct.device)
    mh = m[ti].cpu().numpy()
    rh = np.ascontiguousarray(r[ti].cpu().numpy().view(np.uint32)).view(np.uint64)
    kh = kk[ti].cpu().numpy()

    def u32(t):
        return np.ascontiguousarray(t[ti].cpu().numpy().view(np.uint32))

    want_ct = ck.encrypt(mh, rh, threads)
    got = u32(ct)
    bad = int((got != want_ct.view(np.uint32).reshape(got.shape)).any(axis=1).sum())
    assert bad == 0, f"encrypt parity: {bad} of {idx.size} sampled ciphertexts differ from paillier_z"
    want_cm = ck.mul(np.ascontiguousarray(want_ct), kh, threads)
    got = u32(cm)
    bad = int((got != want_cm.view(np.uint32).reshape(got.shape)).any(axis=1).sum())
    assert bad == 0, f"mul parity: {bad} of {idx.size} sampled ciphertexts differ from paillier_z"
    want_cs = ck.add(np.ascontiguousarray(want_ct), np.ascontiguousarray(u32(ct2)).view(np.uint64), threads)
    got = u32(cs)
    bad = int((got != want_cs.view(np.uint32).reshape(got.shape)).any(axis=1).sum())
    assert bad == 0, f"add parity: {bad} of {idx.size} sampled ciphertexts differ from paillier_z"
    return int(idx.size) * 3


def reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    import numpy as np

    from oracle import cref
    from oracle import paillier_z as pz

    threads = os.cpu_count() or 1
    pk, sk = pz.keygen(KEY_BITS, KEY_SEED)
    ck = cref.CKey(KEY_BITS, pk, sk, window=10)
    ns = 64 * threads
    rng = np.random.default_rng(11)
    m = rng.integers(-(2 ** M_BITS), 2 ** M_BITS, size=ns, dtype=np.int64)
    m2 = rng.integers(-(2 ** M_BITS), 2 ** M_BITS, size=ns, dtype=np.int64)
    r = rng.integers(0, 2 ** 63, size=(ns, ck.r_limbs), dtype=np.int64).astype(np.uint64) * 2 + 1
    k = rng.integers(-(2 ** 63), 2 ** 63 - 1, size=ns, dtype=np.int64)
    ct2 = ck.encrypt(m2, r, threads)

    def step():
        ct = ck.encrypt(m, r, threads)
        cs = ck.add(ct, ct2, threads)
        ck.mul(ct, k, threads)
        d, _ = ck.decrypt(cs, threads)
        return d

    for _ in range(args.warmup):
        d = step()
    assert np.array_equal(d, m + m2)
    t = time.perf_counter()
    for _ in range(args.steps):
        step()
    dt = time.perf_counter() - t
    value = 4 * ns * args.steps / dt
    sample = f"{ns} elements per step (enc+add+mul+dec), paillier_z C restatement, {threads} threads"
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
        "data": "synthetic", "config": {"workload": WORKLOAD, "sample_elements_per_step": ns,
                                        "sample_stands_for": "the 2^20-element step of the same workload: "
                                                            "per-element work is identical, so ops/s compare"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
def ours_arm(args):
    import numpy as np
    import torch

    import heu_gb300 as hg
    from heu_gb300 import capi

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    lib = capi.load()
    n = args.n
    kp = hg.keygen(KEY_BITS, KEY_SEED)
    ctx = hg.Context(local)
    key = ctx.load_key(KEY_BITS, kp["n"], kp["h_s"], kp["p"], kp["q"], table_window=args.window)
    tuned = None
    if args.key_config:
        from heu_gb300 import autotune

        cfg = autotune.get_config(key)
        cfg.update({k: int(v) for k, v in (kv.split("=") for kv in args.key_config.split(","))})
        autotune.set_config(key, cfg)
        tuned = autotune.get_config(key)
    elif not args.no_tune:
        from heu_gb300 import autotune

        tuned, _ = autotune.tune(key, calib=131072)
    S, RL = key.ct_limbs, key.r_limbs
    gen = torch.Generator(device=dev)
    gen.manual_seed(1000 + rank)
    m = torch.randint(-(2 ** M_BITS), 2 ** M_BITS, (n,), dtype=torch.int64, device=dev, generator=gen)
    m2 = torch.randint(-(2 ** M_BITS), 2 ** M_BITS, (n,), dtype=torch.int64, device=dev, generator=gen)
    r = torch.randint(-(2 ** 31), 2 ** 31, (n, RL), dtype=torch.int32, device=dev, generator=gen)
    r2 = torch.randint(-(2 ** 31), 2 ** 31, (n, RL), dtype=torch.int32, device=dev, generator=gen)
    kk = torch.randint(-(2 ** 63), 2 ** 63 - 1, (n,), dtype=torch.int64, device=dev, generator=gen)
    ct = torch.empty((n, S), dtype=torch.int32, device=dev)
    ct2 = torch.empty_like(ct)
    cs = torch.empty_like(ct)
    cm = torch.empty_like(ct)
    d = torch.empty((n,), dtype=torch.int64, device=dev)
    ovf = torch.empty((n,), dtype=torch.uint8, device=dev)
    stream = torch.cuda.Stream(device=dev)
    sp = ctypes.c_void_p(stream.cuda_stream)
    h = ctx.handle

    def P(x):
        return ctypes.c_void_p(x.data_ptr())

    with torch.cuda.stream(stream):
        capi.check(lib.hg_dev_encrypt(h, key.id, P(m2), P(r2), P(ct2), n, sp))
    torch.cuda.synchronize()

    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(5)] for _ in range(args.steps)]

    ops = args.ops
    if "add" not in ops:
        cs.copy_(ct2)  # decrypt then reads the setup ciphertexts (plaintexts m2)

    def step(e=None):
        with torch.cuda.stream(stream):
            if e:
                e[0].record(stream)
            if "encrypt" in ops:
                capi.check(lib.hg_dev_encrypt(h, key.id, P(m), P(r), P(ct), n, sp))
            if e:
                e[1].record(stream)
            if "add" in ops:
                capi.check(lib.hg_dev_add(h, key.id, P(ct), P(ct2), P(cs), n, sp))
            if e:
                e[2].record(stream)
            if "mul" in ops:
                capi.check(lib.hg_dev_mul(h, key.id, P(ct), P(kk), P(cm), n, sp))
            if e:
                e[3].record(stream)
            if "decrypt" in ops:
                capi.check(lib.hg_dev_decrypt(h, key.id, P(cs), P(d), P(ovf), n, sp))
            if e:
                e[4].record(stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    capi.check(lib.hg_dev_check(h))
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clk = ClockSampler(local)
    clk.start()
    launches0 = capi.launch_count()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for i in range(args.steps):
        step(ev[i])
    t1.record(stream)
    torch.cuda.synchronize()
    launches = capi.launch_count() - launches0
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = clk.stop()
    elapsed = t0.elapsed_time(t1) / 1e3
    names = ("encrypt", "add", "mul", "decrypt")
    op_s = {nm: sum(ev[i][j].elapsed_time(ev[i][j + 1]) for i in range(args.steps)) / 1e3
            for j, nm in enumerate(names)}
    if dist:
        t = torch.tensor([elapsed], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed = float(t.item())
    capi.check(lib.hg_dev_check(h))
    # correctness of the timed outputs
    if "decrypt" in ops:
        assert int(ovf.sum().item()) == 0
        want = (m + m2) if ("add" in ops and "encrypt" in ops) else m2
        if "add" in ops or "encrypt" not in ops:
            assert torch.equal(d, want), "decrypt mismatch"
    if "mul" in ops and "encrypt" in ops:
        idx = [0, 1, n // 3, n - 1]
        cm_h = cm[idx].cpu().numpy().view(np.uint32)
        got = key.decrypt_bn(cm_h)
        mh, kh = m[idx].cpu().tolist(), kk[idx].cpu().tolist()
        assert got == [a * b for a, b in zip(mh, kh)], "mul spot check mismatch"

    parity_checked = 0
    if len(ops) == 4 and not args.no_parity:
        parity_checked = parity_sample(kp, m, r, kk, ct, cm, cs, ct2)

    value = len(ops) * n * world * args.steps / elapsed
    per_op = {nm: n * args.steps / op_s[nm] for nm in names if nm in ops}
    if "mul" in ops:
        # the same Mul with |k| (no negative scalar, so no batch inverse):
        # separates the inverse's cost from the exponentiation's
        ka = torch.where(kk == -(2 ** 63), torch.full_like(kk, 2 ** 63 - 1), kk.abs())
        ea = torch.cuda.Event(enable_timing=True)
        eb = torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            capi.check(lib.hg_dev_mul(h, key.id, P(ct), P(ka), P(cm), n, sp))
            ea.record(stream)
            for _ in range(args.steps):
                capi.check(lib.hg_dev_mul(h, key.id, P(ct), P(ka), P(cm), n, sp))
            eb.record(stream)
        torch.cuda.synchronize()
        per_op["mul_nonneg_k"] = n * args.steps / (ea.elapsed_time(eb) / 1e3)
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    mhz = (clocks or {}).get("sm_mhz") or (clocks or {}).get("sm_max_mhz")
    issue_bound = 32 * sms * mhz * 1e6 / 1e12 if mhz else None
    macs_dec = decrypt_macs(KEY_BITS) * n
    dec_avg = op_s["decrypt"] / args.steps
    achieved = macs_dec / dec_avg / 1e12 if "decrypt" in ops else None
    peak_chain = capi.mac_peak(local, 0) / 1e12
    peak_wide = capi.mac_peak(local, 1) / 1e12
    peak = max(peak_chain, peak_wide)
    k_host = kk.cpu().numpy()
    work = {
        "encrypt": encrypt_macs(KEY_BITS, args.window) * n,
        "add": mm_macs(KEY_BITS // 16) * n,
        "mul": mul_macs(KEY_BITS, k_host[: 1 << 14]) * (n / min(n, 1 << 14)),
        "decrypt": macs_dec,
    }
    roof_ops = {nm: work[nm] / (op_s[nm] / args.steps) / 1e12 for nm in names if nm in ops}
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath):
        try:
            tj = json.load(open(tpath))
            traffic = tj.get("decrypt_bytes_per_ciphertext", None)
            if traffic is not None:
                traffic = traffic * n
        except (OSError, ValueError):
            traffic = None

    # ---- e2e through the host-pointer C-ABI ------------------------------
    e2e = None
    if not args.no_e2e:
        pin = dict(pin_memory=True)
        m_h = m.cpu().pin_memory()
        r_h = r.cpu().pin_memory()
        k_h = kk.cpu().pin_memory()
        ct2_h = ct2.cpu().pin_memory()
        ct_h = torch.empty((n, S), dtype=torch.int32, **pin)
        cs_h = torch.empty((n, S), dtype=torch.int32, **pin)
        cm_hh = torch.empty((n, S), dtype=torch.int32, **pin)
        d_h = torch.empty((n,), dtype=torch.int64, **pin)
        o_h = torch.empty((n,), dtype=torch.uint8, **pin)

        e2e_op_s = {"encrypt": 0.0, "add": 0.0, "mul": 0.0, "decrypt": 0.0}
        e2e_trace = []

        def e2e_step():
            t = time.perf_counter()
            capi.check(lib.hg_encrypt(h, key.id, P(m_h), P(r_h), P(ct_h), n))
            t1 = time.perf_counter()
            capi.check(lib.hg_add(h, key.id, P(ct_h), P(ct2_h), P(cs_h), n))
            t2 = time.perf_counter()
            capi.check(lib.hg_mul(h, key.id, P(ct_h), P(k_h), P(cm_hh), n))
            t3 = time.perf_counter()
            capi.check(lib.hg_decrypt(h, key.id, P(cs_h), P(d_h), P(o_h), n))
            t4 = time.perf_counter()
            for nm, dt in zip(("encrypt", "add", "mul", "decrypt"), (t1 - t, t2 - t1, t3 - t2, t4 - t3)):
                e2e_op_s[nm] += dt
            e2e_trace.append([round(t1 - t, 4), round(t2 - t1, 4), round(t3 - t2, 4), round(t4 - t3, 4)])

        e2e_step()
        for nm in e2e_op_s:
            e2e_op_s[nm] = 0.0
        if dist:
            dist.barrier()
        t = time.perf_counter()
        for _ in range(args.e2e_steps):
            e2e_step()
        e2e_dt = time.perf_counter() - t
        # raw pinned copy bandwidth on this host, for reading the e2e overhead
        big = torch.empty((n, S), dtype=torch.int32, pin_memory=True)
        dbig = torch.empty((n, S), dtype=torch.int32, device=dev)
        torch.cuda.synchronize()
        tc = time.perf_counter()
        dbig.copy_(big, non_blocking=True)
        torch.cuda.synchronize()
        h2d_gbs = big.numel() * 4 / (time.perf_counter() - tc) / 1e9
        tc = time.perf_counter()
        big.copy_(dbig, non_blocking=True)
        torch.cuda.synchronize()
        d2h_gbs = big.numel() * 4 / (time.perf_counter() - tc) / 1e9
        del big, dbig
        # the same copies as the engine's runtime sees them
        seen = {}
        for nm, buf, dr in (("ct_in_h2d", ct2_h, 0), ("ct_out_d2h", cs_h, 1)):
            mt, g = ctypes.c_int(), ctypes.c_double()
            rc = lib.hg_probe_host_copy(local, P(buf), buf.numel() * 4, dr, ctypes.byref(mt), ctypes.byref(g))
            seen[nm] = {"rc": rc, "mem_type": mt.value, "gbs": g.value}
        if dist:
            tt = torch.tensor([e2e_dt], device=dev, dtype=torch.float64)
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
            e2e_dt = float(tt.item())
        assert torch.equal(d_h, (m + m2).cpu()), "e2e decrypt mismatch"
        assert len(ops) == 4, "e2e runs the full step"
        cb = S * 4
        h2d = n * (8 + RL * 4) + n * 2 * cb + n * (cb + 8) + n * cb
        d2h = n * cb * 3 + n * 9
        e2e = {"value": 4 * n * world * args.e2e_steps / e2e_dt, "unit": UNIT, "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "steps": args.e2e_steps,
               "api": "hg_encrypt/hg_add/hg_mul/hg_decrypt (host pointers, pinned)",
               "per_op_s": {k: v / args.e2e_steps for k, v in e2e_op_s.items()},
               "trace_s": e2e_trace,
               "pinned_copy_gbs": {"h2d": h2d_gbs, "d2h": d2h_gbs, "engine_runtime": seen}}

    # per-call latency of small host-pointer calls (no per-call allocation:
    # staging buffers and streams belong to the context)
    small = {}
    if not args.no_e2e:
        for cnt in (1, 16, 256, 4096):
            mh = m[:cnt].cpu().numpy()
            rh = r[:cnt].cpu().numpy().view(np.uint32)
            cth = np.empty((cnt, S), np.uint32)
            dh = np.empty(cnt, np.int64)
            oh = np.empty(cnt, np.uint8)
            ts = {"encrypt": [], "decrypt": []}
            for it in range(12):
                t = time.perf_counter()
                capi.check(lib.hg_encrypt(h, key.id, ctypes.c_void_p(mh.ctypes.data), ctypes.c_void_p(rh.ctypes.data),
                                          ctypes.c_void_p(cth.ctypes.data), cnt))
                t2 = time.perf_counter()
                capi.check(lib.hg_decrypt(h, key.id, ctypes.c_void_p(cth.ctypes.data), ctypes.c_void_p(dh.ctypes.data),
                                          ctypes.c_void_p(oh.ctypes.data), cnt))
                t3 = time.perf_counter()
                if it >= 2:
                    ts["encrypt"].append((t2 - t) * 1e6)
                    ts["decrypt"].append((t3 - t2) * 1e6)
            assert np.array_equal(dh, mh), "small-call decrypt mismatch"
            small[str(cnt)] = {k: float(np.median(v)) for k, v in ts.items()}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        rates, step_rate, cores, sample = cpu_sample()
        cpu = {"value": step_rate, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample,
               "per_op": rates}

    extras = {}
    if rank == 0 and world == 1 and not args.no_extras:
        # the rest of the metric, outside the timed step: reductions (config 3),
        # the uneven batch against plain calls (config 4), the served stream at
        # a sub-capacity and a saturating rate (config 5); each in its own
        # context once this one has released its table
        ctx.close()
        ctx = None
        extras = run_extras(args)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": elapsed / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "key_bits": KEY_BITS, "batch": n, "table_window": args.window,
                       "autotuned": tuned,
                       "l2": "inputs larger than L2 (512 MiB per ciphertext array); no flush",
                       "parallelism": f"replicas x{world}"},
            "per_op_ops_per_s": per_op,
            "per_op_note": (f"encrypt uses a fixed-base table of window {args.window} "
                            f"({encrypt_macs(KEY_BITS, args.window) // mm_macs(KEY_BITS // 16)} Montgomery "
                            "multiplications per ciphertext, a time-memory trade of the 280 GB HBM) where the "
                            "CPU restatement uses HEU's window 10 (105); the other ops run the same algorithms "
                            "on both sides"),
            "roofline": {"bound": "imad", "kernel": "decrypt (CRT, k_decrypt)", "achieved": achieved,
                         "peak": peak, "unit": "TMAC/s", "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                         "peak_source": "measured live: hg_probe_mac_peak (best of mad.wide / carry-chain "
                                        "patterns); MEASURED_PEAKS.json has no integer figure",
                         "peak_chain_pattern": peak_chain, "peak_wide_pattern": peak_wide,
                         # the issue bound of the wide multiply-add: 4 cycles per warp
                         # instruction on each SM sub-partition's fmaheavy pipe = 32 MACs per
                         # clock per SM, at the SM clock sampled during the timed region
                         "issue_bound": issue_bound, "frac_of_issue_bound": (achieved / issue_bound)
                         if (achieved and issue_bound) else None,
                         "per_op_tmacs": roof_ops},
            "parity_checked": parity_checked,
            "parity": ("strided sample of the timed Encrypt / Add / Mul outputs byte-equal (Montgomery form) to "
                       "the paillier_z C restatement given the same m, r, k; every timed decryption equal to "
                       "m + m2"),
            "e2e": e2e,
            "small_call_us": small,
            "cpu_baseline": cpu,
            "gpu_launches": launches,
            "clocks": clocks,
        }
        line.update(extras)
        if "reductions" in extras:
            per_op["sum"] = extras["reductions"]["sum"]["units_per_s"]
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    if ctx is not None:
        ctx.close()
    return 0


def run_extras(args):
    """Summaries of configs 3, 4 and 5 for the default line (each measured
    with CUDA events or wall clocks in its own context, after the main step's
    timed region)."""
    out = {}
    c3 = c3_measure(args, 2, 1)
    out["reductions"] = {k: {"seconds": v["seconds"], "units_per_s": v["units_per_s"],
                             "algorithmic_tmacs": v["algorithmic_tmacs"], "hbm_gbs": v["hbm_gbs"]}
                         for k, v in c3["results"].items()}
    out["reductions"]["config"] = c3["config"]
    c4 = c4_measure(args, 2, 1)
    out["batched_vs_plain"] = {"batched_over_plain": c4["batched_over_plain"],
                               "batched_ops_per_s": c4["value"], "plain_ops_per_s": c4["plain_per_call_ops_per_s"],
                               "steps": c4["steps"], "config": c4["config"]}
    c5 = c5_measure(args, [20, 50, 3000], lambda rate: 250 if rate <= 100 else 1000)
    out["serve"] = {"served_over_plain": c5["served_over_plain"], "plain_ops_per_s": c5["plain_per_call_ops_per_s"],
                    "rates": c5["rates"], "config": c5["config"]}
    return out


# ---------------------------------------------------------------------------
def _load_keys(ctx, spec, tune):
    """spec: list of (bits, seed, table_window) -> loaded keys (tuned if asked)."""
    import heu_gb300 as hg
    from heu_gb300 import autotune

    keys = []
    for bits, seed, w in spec:
        kp = hg.keygen(bits, seed)
        key = ctx.load_key(bits, kp["n"], kp["h_s"], kp["p"], kp["q"], table_window=w)
        if tune:
            autotune.tune(key, calib=131072)
        keys.append(key)
    return keys


def c4_arm(args):
    """Config 4: 64 uneven jobs over 1024/2048/3072-bit keys (lengths
    log-uniform in [16, 262144], op mix 40% encrypt / 30% mul / 20% add / 10%
    decrypt, int64 plaintexts and scalars uniform), run as one persistent
    launch replayed from a CUDA graph, against the plain per-call kernels."""
    print(json.dumps(c4_measure(args, args.steps, args.warmup)), flush=True)
    return 0


def c4_measure(args, steps, warmup):
    import numpy as np
    import torch

    import heu_gb300 as hg
    from heu_gb300 import capi
    from heu_gb300.batch import ADD, DECRYPT, ENCRYPT, MUL

    dev = torch.device("cuda", 0)
    ctx = hg.Context(0)
    lib, h = ctx.lib, ctx.handle
    keys = _load_keys(ctx, [(1024, 1, 16), (2048, 0, 16), (3072, 2, 14)], not args.no_tune)
    rng = np.random.default_rng(4)
    gen = torch.Generator(device=dev)
    gen.manual_seed(44)
    ops_p = [0.4, 0.3, 0.2, 0.1]
    op_codes = [ENCRYPT, MUL, ADD, DECRYPT]
    jobs = []
    total = 0
    for _ in range(64):
        key = keys[int(rng.integers(3))]
        n = int(np.floor(np.exp(rng.uniform(np.log(16), np.log(262144)))))
        op = op_codes[int(rng.choice(4, p=ops_p))]
        S, RL = key.ct_limbs, key.r_limbs
        m = torch.randint(-(2 ** 63), 2 ** 63 - 1, (n,), dtype=torch.int64, device=dev, generator=gen)
        r = torch.randint(-(2 ** 31), 2 ** 31, (n, RL), dtype=torch.int32, device=dev, generator=gen)
        base = torch.empty((n, S), dtype=torch.int32, device=dev)
        capi.check(lib.hg_dev_encrypt(h, key.id, ctypes.c_void_p(m.data_ptr()), ctypes.c_void_p(r.data_ptr()),
                                      ctypes.c_void_p(base.data_ptr()), n, None))
        torch.cuda.synchronize()  # torch's stream reads `base` below; the engine's stream wrote it
        j = dict(key=key, n=n, op=op, m=m, r=r, base=base)
        if op == MUL:
            j["k"] = torch.randint(-(2 ** 63), 2 ** 63 - 1, (n,), dtype=torch.int64, device=dev, generator=gen)
        if op == ADD:
            j["other"] = base.roll(1, 0).contiguous()
        if op == DECRYPT:
            j["out_p"] = torch.empty((n,), dtype=torch.int64, device=dev)
            j["out_b"] = torch.empty((n,), dtype=torch.int64, device=dev)
            j["ovf"] = torch.empty((n,), dtype=torch.uint8, device=dev)
        else:
            j["out_p"] = torch.empty((n, S), dtype=torch.int32, device=dev)
            j["out_b"] = torch.empty((n, S), dtype=torch.int32, device=dev)
        jobs.append(j)
        total += n
    torch.cuda.synchronize()
    stream = torch.cuda.Stream(device=dev)
    sp = ctypes.c_void_p(stream.cuda_stream)

    def P(t):
        return ctypes.c_void_p(t.data_ptr())

    def plain():
        for j in jobs:
            kid, n = j["key"].id, j["n"]
            if j["op"] == ENCRYPT:
                capi.check(lib.hg_dev_encrypt(h, kid, P(j["m"]), P(j["r"]), P(j["out_p"]), n, sp))
            elif j["op"] == MUL:
                capi.check(lib.hg_dev_mul(h, kid, P(j["base"]), P(j["k"]), P(j["out_p"]), n, sp))
            elif j["op"] == ADD:
                capi.check(lib.hg_dev_add(h, kid, P(j["base"]), P(j["other"]), P(j["out_p"]), n, sp))
            else:
                capi.check(lib.hg_dev_decrypt(h, kid, P(j["base"]), P(j["out_p"]), P(j["ovf"]), n, sp))

    batch = hg.Batch(ctx)
    for j in jobs:
        if j["op"] == ENCRYPT:
            batch.add(j["key"], ENCRYPT, j["n"], j["m"], j["r"], j["out_b"])
        elif j["op"] == MUL:
            batch.add(j["key"], MUL, j["n"], j["base"], j["k"], j["out_b"])
        elif j["op"] == ADD:
            batch.add(j["key"], ADD, j["n"], j["base"], j["other"], j["out_b"])
        else:
            batch.add(j["key"], DECRYPT, j["n"], j["base"], None, j["out_b"], j["ovf"])
    # batch variant: the fastest of the two layout sets and each key's tuned
    # layout (one launch per set in use) on one eager run
    best_v, best_t = 0, None
    for v in (0, 1, hg.batch.PER_KEY):
        batch.set_variant(v)
        batch.run(stream=stream)
        batch.wait(stream=stream)
        t0 = time.perf_counter()
        batch.run(stream=stream)
        batch.wait(stream=stream)
        dt = time.perf_counter() - t0
        if best_t is None or dt < best_t:
            best_v, best_t = v, dt
    batch.set_variant(best_v)

    def timed(fn, steps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
            for _ in range(steps):
                fn()
            e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1e3

    for _ in range(warmup):
        plain()
        batch.run(stream=stream, graph=True)
    batch.wait(stream=stream)
    capi.check(lib.hg_dev_check(h))
    t_plain = timed(plain, steps)
    launches0 = capi.launch_count()
    t_batch = timed(lambda: batch.run(stream=stream, graph=True), steps)
    launches = capi.launch_count() - launches0
    batch.wait(stream=stream)
    capi.check(lib.hg_dev_check(h))
    for j in jobs:
        assert torch.equal(j["out_p"], j["out_b"]), "batched result differs from per-call result"
        if j["op"] == DECRYPT:
            assert torch.equal(j["out_b"], j["m"])
    mix = {}
    for j in jobs:
        nm = {ENCRYPT: "encrypt", MUL: "mul", ADD: "add", DECRYPT: "decrypt"}[j["op"]]
        mix[f"{nm}_{j['key'].key_bits}"] = mix.get(f"{nm}_{j['key'].key_bits}", 0) + j["n"]
    line = {
        "metric": "Paillier ops/s, 64 uneven jobs over 1024/2048/3072-bit keys (config 4), batched vs plain GPU",
        "value": total * steps / t_batch, "unit": UNIT, "n_gpus": 1, "steps": steps,
        "warmup": warmup, "ms_per_step": t_batch / steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": {"workload": "config4", "jobs": 64, "elements_per_step": total, "mix": mix,
                   "batch_variant": "per_key" if best_v == hg.batch.PER_KEY else best_v, "graph": True},
        "plain_per_call_ops_per_s": total * steps / t_plain,
        "batched_over_plain": t_plain / t_batch,
        "gpu_launches": launches,
    }
    batch.close()
    ctx.close()
    return line


def c3_arm(args):
    """Config 3: heu.numpy reductions with a 2048-bit key on fixed-point
    gradients (N(0,1) * 2^20): Sum of 2^20 ciphertexts, FeatureWiseBucketSum
    over 64 features x 256 buckets, MatMul 4096x256 ciphertexts @ 256x64
    int32 in [-2^15, 2^15)."""
    print(json.dumps(c3_measure(args, args.steps, args.warmup)), flush=True)
    return 0


def c3_measure(args, steps, warmup):
    import numpy as np
    import torch

    import heu_gb300 as hg
    from heu_gb300 import capi

    dev = torch.device("cuda", 0)
    ctx = hg.Context(0)
    lib, h = ctx.lib, ctx.handle
    key = _load_keys(ctx, [(2048, 0, 16)], not args.no_tune)[0]
    rng = np.random.default_rng(5)
    n, F, B = 1 << 20, 64, 256
    M, K, N = 4096, 256, 64
    g = torch.from_numpy(np.round(rng.standard_normal(n) * (1 << 20)).astype(np.int64)).to(dev)
    r = torch.randint(-(2 ** 31), 2 ** 31, (n, key.r_limbs), dtype=torch.int32, device=dev)
    ct = torch.empty((n, key.ct_limbs), dtype=torch.int32, device=dev)

    def P(t):
        return ctypes.c_void_p(t.data_ptr())

    capi.check(lib.hg_dev_encrypt(h, key.id, P(g), P(r), P(ct), n, None))
    torch.cuda.synchronize()  # the reductions below run on another stream
    om = torch.from_numpy(rng.integers(0, B, size=(n, F)).astype(np.uint8)).to(dev)
    bsum = torch.empty((F * B, key.ct_limbs), dtype=torch.int32, device=dev)
    s1 = torch.empty((1, key.ct_limbs), dtype=torch.int32, device=dev)
    y = rng.integers(-(2 ** 15), 2 ** 15, size=(K, N), dtype=np.int64)
    mm = torch.empty((M * N, key.ct_limbs), dtype=torch.int32, device=dev)
    stream = torch.cuda.Stream(device=dev)
    sp = ctypes.c_void_p(stream.cuda_stream)
    yc = np.ascontiguousarray(y)

    def run_sum():
        capi.check(lib.hg_dev_sum(h, key.id, P(ct), n, P(s1), sp))

    def run_bucket():
        capi.check(lib.hg_dev_bucket_sum(h, key.id, P(ct), n, 1, P(om), F, B, 0, P(bsum), sp))

    def run_matmul():
        capi.check(lib.hg_dev_matmul(h, key.id, P(ct), M, K, ctypes.c_void_p(yc.ctypes.data), N, P(mm), sp))

    res = {}
    cb = key.ct_limbs * 4
    # --ops may name a subset of the reductions (profiling one kernel)
    chosen = [o for o in getattr(args, "ops", []) if o in ("sum", "bucket_sum", "matmul")]
    for name, fn, units, macs_per_unit, nbytes in (
            ("sum", run_sum, n, mm_macs(128), n * cb + cb),
            ("bucket_sum", run_bucket, n * F, mm_macs(128), n * cb + n * F + F * B * cb),
            ("matmul", run_matmul, M * N, (K + 16) * mm_macs(128), M * K * cb + K * N * 8 + M * N * cb)):
        if chosen and name not in chosen:
            continue
        for _ in range(max(1, warmup)):
            fn()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
            for _ in range(steps):
                fn()
            e1.record(stream)
        torch.cuda.synchronize()
        dt = e0.elapsed_time(e1) / 1e3 / steps
        res[name] = {"seconds": dt, "units_per_s": units / dt, "algorithmic_tmacs": units * macs_per_unit / dt / 1e12,
                     "algorithmic_bytes": nbytes, "hbm_gbs": nbytes / dt / 1e9}
    capi.check(lib.hg_dev_check(h))
    # correctness through decryption
    key_dec = lambda t: key.decrypt(t.cpu().numpy().view(np.uint32))  # noqa: E731
    gh, omh = g.cpu().numpy(), om.cpu().numpy()
    if "sum" in res:
        dsum, _ = key_dec(s1)
        assert int(dsum[0]) == int(g.sum().item())
    if "bucket_sum" in res:
        db, _ = key_dec(bsum)
        exact = np.zeros((F, B), dtype=np.int64)
        for f in range(F):
            np.add.at(exact[f], omh[:, f], gh)
        assert np.array_equal(db.reshape(F, B), exact)
    if "matmul" in res:
        dm, _ = key_dec(mm)
        assert np.array_equal(dm.reshape(M, N), gh[: M * K].reshape(M, K) @ y)
    peak = max(capi.mac_peak(0, 0), capi.mac_peak(0, 1)) / 1e12
    line = {
        "metric": "heu.numpy reductions on 2048-bit ciphertexts (config 3): Sum, bucket-sum, MatMul",
        "value": res[next(iter(res))]["units_per_s"] if "bucket_sum" not in res else res["bucket_sum"]["units_per_s"],
        "unit": "ciphertext-products/s (bucket-sum)" if "bucket_sum" in res else "units/s (%s)" % next(iter(res)),
        "n_gpus": 1, "steps": steps, "warmup": warmup, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": {"workload": "config3", "sum_n": n, "bucket_sum": [n, F, B], "matmul": [M, K, N]},
        "results": res, "mac_peak_tmacs": peak,
    }
    ctx.close()
    return line


def ou_arm(args):
    """Okamoto-Uchiyama (HEU's ou scheme) on one GB300: 2048-bit key from
    seed 0, 2^20 int64 plaintexts in [-2^40, 2^40), r < 2^110; one step =
    Encrypt + Add + Mul (64-bit k) + Decrypt over the batch, with the OU
    oracle timed on a bounded sample on one host core."""
    import numpy as np
    import torch

    import heu_gb300 as hg
    import heu_gb300.engine as eng
    from heu_gb300 import capi

    dev = torch.device("cuda", 0)
    kp = eng.ou_keygen(2048, 0)
    ctx = hg.Context(0)
    key = ctx.load_ou_key(2048, kp["n"], kp["G"], kp["H"], kp["max_pt_bits"], kp["p"], kp["q"], kp["t"],
                          kp["gp_inv"], table_window=16)
    lib, h = ctx.lib, ctx.handle
    n, S = args.n, key.ct_limbs
    gen = torch.Generator(device=dev)
    gen.manual_seed(21)
    m = torch.randint(-(2 ** M_BITS), 2 ** M_BITS, (n,), dtype=torch.int64, device=dev, generator=gen)
    r = torch.randint(-(2 ** 31), 2 ** 31, (n, key.r_limbs), dtype=torch.int32, device=dev, generator=gen)
    r[:, 3] &= (1 << (110 - 96)) - 1
    kk = torch.randint(-(2 ** 63), 2 ** 63 - 1, (n,), dtype=torch.int64, device=dev, generator=gen)
    ct = torch.empty((n, S), dtype=torch.int32, device=dev)
    cs = torch.empty_like(ct)
    cm = torch.empty_like(ct)
    d = torch.empty((n,), dtype=torch.int64, device=dev)
    ovf = torch.empty((n,), dtype=torch.uint8, device=dev)
    st = torch.cuda.Stream(device=dev)
    sp = ctypes.c_void_p(st.cuda_stream)

    def P(t):
        return ctypes.c_void_p(t.data_ptr())

    names = ("encrypt", "add", "mul", "decrypt")
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(5)] for _ in range(max(args.steps, 1))]

    def step(e=None):
        with torch.cuda.stream(st):
            e and e[0].record(st)
            capi.check(lib.hg_dev_encrypt(h, key.id, P(m), P(r), P(ct), n, sp))
            e and e[1].record(st)
            capi.check(lib.hg_dev_add(h, key.id, P(ct), P(ct), P(cs), n, sp))
            e and e[2].record(st)
            capi.check(lib.hg_dev_mul(h, key.id, P(ct), P(kk), P(cm), n, sp))
            e and e[3].record(st)
            capi.check(lib.hg_dev_decrypt(h, key.id, P(cs), P(d), P(ovf), n, sp))
            e and e[4].record(st)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    capi.check(lib.hg_dev_check(h))
    clk = ClockSampler(0)
    clk.start()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(st)
    for i in range(args.steps):
        step(ev[i])
    t1.record(st)
    torch.cuda.synchronize()
    clocks = clk.stop()
    capi.check(lib.hg_dev_check(h))
    assert int(ovf.sum().item()) == 0 and torch.equal(d, 2 * m), "OU decrypt mismatch"
    elapsed = t0.elapsed_time(t1) / 1e3
    op_s = {nm: sum(ev[i][j].elapsed_time(ev[i][j + 1]) for i in range(args.steps)) / 1e3 / args.steps
            for j, nm in enumerate(names)}
    w, wd = 16, 5
    t_bits = kp["t"].bit_length()
    work = {
        "encrypt": (-(-64 // w) + -(-110 // w)) * mm_macs(S) * n,
        "add": mm_macs(S) * n,
        "mul": mul_macs(2048, kk[: 1 << 14].cpu().numpy()) * (n / min(n, 1 << 14)),
        "decrypt": ((t_bits - 1) + -(-t_bits // (wd + 1)) + 2 ** (wd - 1) + 3) * mm_macs(64) * n,
    }
    peak = max(capi.mac_peak(0, 0), capi.mac_peak(0, 1)) / 1e12
    tmacs = {nm: work[nm] / op_s[nm] / 1e12 for nm in names}
    # the OU oracle on one host core, bounded sample
    from oracle import ou
    from oracle.prg import Prg

    pk = ou.PublicKey(kp["n"], kp["G"], kp["H"], 1 << kp["max_pt_bits"])
    sk = ou.SecretKey(kp["p"], kp["q"], kp["t"], kp["gp_inv"])
    prg = Prg(5)
    ns = 400
    ms = [prg.int64_uniform(-(2 ** M_BITS), 2 ** M_BITS) for _ in range(ns)]
    rs = [prg.randbits(110) for _ in range(ns)]
    ks = [prg.int64_uniform(-(2 ** 63), 2 ** 63) for _ in range(ns)]
    rates = {}
    t = time.perf_counter()
    zs = [ou.encrypt(pk, a, b) for a, b in zip(ms, rs)]
    rates["encrypt"] = ns / (time.perf_counter() - t)
    t = time.perf_counter()
    ss = [ou.add(pk, z, z) for z in zs]
    rates["add"] = ns / (time.perf_counter() - t)
    t = time.perf_counter()
    [ou.mul(pk, z, k) for z, k in zip(zs[:100], ks[:100])]
    rates["mul"] = 100 / (time.perf_counter() - t)
    t = time.perf_counter()
    dd = [ou.decrypt(pk, sk, z) for z in ss[:200]]
    rates["decrypt"] = 200 / (time.perf_counter() - t)
    assert dd == [2 * a for a in ms[:200]]
    cpu_rate = 4.0 / sum(1.0 / rates[o] for o in names)
    line = {
        "metric": "OU-2048 ops/s (enc/add/mul/dec)", "value": 4 * n * args.steps / elapsed, "unit": UNIT,
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": elapsed / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": {"workload": "ou: 2048-bit OU key (n of %d bits), 2^20 int64 m~U[-2^40,2^40), r<2^110, "
                               "enc+add+mul(64-bit k)+dec per step" % kp["n"].bit_length(),
                   "table_window": w, "ciphertext_limbs": S},
        "per_op_ops_per_s": {nm: n / op_s[nm] for nm in names},
        "roofline": {"bound": "imad", "unit": "TMAC/s", "per_op_tmacs": tmacs, "peak": peak,
                     "frac": {nm: tmacs[nm] / peak for nm in names}},
        "cpu_baseline": {"value": cpu_rate, "unit": UNIT, "cores": 1, "kind": "port", "per_op": rates,
                         "sample": f"OU oracle (Python integers), {ns} enc/add, 100 mul, 200 dec, one core"},
        "clocks": clocks,
    }
    print(json.dumps(line), flush=True)
    ctx.close()
    return 0


def wire_arm(args):
    """HEU wire format (numpy/matrix.h Serialize / LoadFrom) of 2^20
    ciphertexts of a 2048-bit key: GPU pack from device ciphertexts to device
    bytes, and load from host bytes (as received from a peer) to device
    ciphertexts; the host-buffer round trip as e2e; the wire oracle on one
    host core as the CPU baseline.  Roofline: algorithmic HBM bytes of a pack
    (ciphertexts read once, items written once) over the pack's device time."""
    import numpy as np
    import torch

    import heu_gb300 as hg
    import heu_gb300.engine as eng
    from heu_gb300 import capi

    dev = torch.device("cuda", 0)
    kp = eng.keygen(KEY_BITS, KEY_SEED)
    ctx = hg.Context(0)
    key = ctx.load_key(KEY_BITS, kp["n"], kp["h_s"], kp["p"], kp["q"], table_window=12)
    lib, h = ctx.lib, ctx.handle
    n, S = args.n, key.ct_limbs
    gen = torch.Generator(device=dev)
    gen.manual_seed(31)
    m = torch.randint(-(2 ** M_BITS), 2 ** M_BITS, (n,), dtype=torch.int64, device=dev, generator=gen)
    r = torch.randint(-(2 ** 31), 2 ** 31, (n, key.r_limbs), dtype=torch.int32, device=dev, generator=gen)
    ct = torch.empty((n, S), dtype=torch.int32, device=dev)
    back = torch.empty_like(ct)
    st = torch.cuda.Stream(device=dev)
    sp = ctypes.c_void_p(st.cuda_stream)

    def P(t):
        return ctypes.c_void_p(t.data_ptr())

    with torch.cuda.stream(st):
        capi.check(lib.hg_dev_encrypt(h, key.id, P(m), P(r), P(ct), n, sp))
    torch.cuda.synchronize()
    bound = ctypes.c_size_t()
    capi.check(lib.hg_serialize_bound(h, key.id, n, ctypes.byref(bound)))
    dbuf = torch.empty(bound.value, dtype=torch.uint8, device=dev)
    ln = ctypes.c_size_t()
    rows, cols, nd = ctypes.c_size_t(), ctypes.c_size_t(), ctypes.c_int()

    def pack():
        capi.check(lib.hg_dev_serialize(h, key.id, P(ct), n, 1, 1, 1, P(dbuf), bound.value, ctypes.byref(ln), sp))

    pack()
    hbuf = dbuf[:ln.value].cpu().pin_memory()

    def load():
        capi.check(lib.hg_dev_deserialize(h, key.id, P(hbuf), hbuf.numel(), 1, P(back), n, ctypes.byref(rows),
                                          ctypes.byref(cols), ctypes.byref(nd), sp))

    for _ in range(args.warmup):
        pack()
        load()
    torch.cuda.synchronize()
    capi.check(lib.hg_dev_check(h))
    clk = ClockSampler(0)
    clk.start()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    t_pack = t_load = 0.0
    for _ in range(args.steps):
        ev[0].record(st)
        pack()
        ev[1].record(st)
        load()
        ev[2].record(st)
        torch.cuda.synchronize()
        t_pack += ev[0].elapsed_time(ev[1]) / 1e3
        t_load += ev[1].elapsed_time(ev[2]) / 1e3
    clocks = clk.stop()
    capi.check(lib.hg_dev_check(h))
    assert torch.equal(back, ct), "wire round trip mismatch"
    t_pack /= args.steps
    t_load /= args.steps
    nbytes = ln.value
    # e2e: host ciphertexts -> host bytes -> host ciphertexts through the C-ABI host-pointer calls
    ct_pin = ct.cpu().pin_memory()
    out_pin = torch.empty(bound.value, dtype=torch.uint8).pin_memory()
    back_pin = torch.empty_like(ct_pin).pin_memory()

    def e2e_step():
        capi.check(lib.hg_serialize(h, key.id, P(ct_pin), n, 1, 1, 1, P(out_pin), bound.value, ctypes.byref(ln)))
        capi.check(lib.hg_deserialize(h, key.id, P(out_pin), ln.value, 1, P(back_pin), n, ctypes.byref(rows),
                                      ctypes.byref(cols), ctypes.byref(nd)))

    e2e_step()
    t = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    t_e2e = (time.perf_counter() - t) / args.steps
    assert torch.equal(back_pin, ct_pin)
    ct_h = ct_pin.numpy().view(np.uint32)
    # the wire oracle on one core, bounded sample
    from oracle import wire

    ns = min(n, 1 << 15)
    vals = hg.limbs_to_ints(ct_h[:ns])
    t = time.perf_counter()
    ob = wire.serialize_matrix(vals, ns, 1, 1, wire.SCHEMA_ZPAILLIER)
    t_os = time.perf_counter() - t
    t = time.perf_counter()
    parsed = wire.parse_matrix(ob)
    t_ol = time.perf_counter() - t
    assert parsed[3] == vals
    algo = n * S * 4 + nbytes  # algorithmic: ciphertexts read once, items written once
    peak = None
    try:
        peak = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"]
    except (OSError, ValueError, KeyError):
        peak = 6800.0
    line = {
        "metric": "HEU wire format ciphertexts/s (serialize + load, 2048-bit)", "value": n / (t_pack + t_load),
        "unit": "ciphertexts/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": (t_pack + t_load) * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u8", "data": "synthetic",
        "config": {"workload": "wire: 2^20 ciphertexts of a 2048-bit key, DenseMatrix msgpack layout, "
                               "pack device->device, load host bytes->device", "bytes": nbytes},
        "per_op_ciphertexts_per_s": {"serialize": n / t_pack, "load": n / t_load},
        "roofline": {"bound": "hbm", "kernel": "serialize (k_wire_sizes + scan + k_wire_write)",
                     "achieved": algo / t_pack / 1e9, "peak": peak, "unit": "GB/s",
                     "frac": algo / t_pack / 1e9 / peak, "traffic": None,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs"},
        "e2e": {"value": n / t_e2e, "unit": "ciphertexts/s", "h2d_bytes_per_step": n * S * 4 + nbytes,
                "d2h_bytes_per_step": nbytes + n * S * 4, "api": "hg_serialize + hg_deserialize (host buffers)"},
        "cpu_baseline": {"value": ns / (t_os + t_ol), "unit": "ciphertexts/s", "cores": 1, "kind": "port",
                         "sample": f"wire oracle (Python) serialize + parse of {ns} ciphertexts, one core"},
        "clocks": clocks,
    }
    print(json.dumps(line), flush=True)
    ctx.close()
    return 0


def c5_arm(args):
    """Config 5: served request stream.  8 resident keypairs (six 2048-bit,
    two 3072-bit), Poisson arrivals at swept rates, lengths log-uniform in
    [1, 65536], op mix encrypt/add/mul/sum/decrypt 30/20/25/15/10, resident
    ciphertext vectors, 40 GB device budget; p50/p99 latency and throughput
    per rate, against the same mix through plain per-call kernels."""
    rates = [20, 50, 100, 300, 1000, 3000, 10000, 50000] if not args.quick else [50, 3000]
    if args.rates:
        rates = [int(v) for v in args.rates.split(",")]
    print(json.dumps(c5_measure(args, rates, lambda rate: min(1000, max(200, int(rate * 3))))), flush=True)
    return 0


OP_NAMES = ("encrypt", "decrypt", "add", "mul", "sum")


def _latency_classes(lat, ops, lens, short_len):
    """p50/p99 (ms) by class: all, short (<= short_len elements) split into
    decrypt and the other ops, per op among the short ones, and long."""
    import numpy as np

    def pct(mask):
        if not mask.any():
            return None
        v = lat[mask] * 1e3
        return {"requests": int(mask.sum()), "p50_ms": float(np.percentile(v, 50)),
                "p99_ms": float(np.percentile(v, 99)), "max_ms": float(v.max())}

    short = lens <= short_len
    out = {"short_le_%d" % short_len: pct(short),
           "short_enc_add_sum": pct(short & ((ops == 0) | (ops == 2) | (ops == 4))),
           "short_non_decrypt": pct(short & (ops != 1)),
           "short_decrypt": pct(short & (ops == 1)),
           "long": pct(~short)}
    out["short_by_op"] = {OP_NAMES[o]: pct(short & (ops == o)) for o in range(5)}
    return out


def _phase_p99(phases, ops, lens, short_len):
    import numpy as np

    m = (lens <= short_len) & (ops != 1)
    if not m.any():
        return None
    names = ("queued", "staged", "gpu_and_retire")
    return {nm: float(np.percentile(phases[m, k], 99) * 1e3) for k, nm in enumerate(names)}


def c5_measure(args, rates, nreq_for_rate):
    import numpy as np
    import torch

    import heu_gb300 as hg
    from heu_gb300 import autotune, capi

    dev = torch.device("cuda", 0)
    ctx = hg.Context(0)
    lib, h = ctx.lib, ctx.handle
    spec = [(2048, s, 16) for s in range(6)] + [(3072, 10 + s, 14) for s in range(2)]
    keys = _load_keys(ctx, spec, False)
    if not args.no_tune:
        c2048, _ = autotune.tune(keys[0], calib=131072)
        c3072, _ = autotune.tune(keys[6], calib=65536)
        for kk in keys[1:6]:
            autotune.set_config(kk, c2048)
        autotune.set_config(keys[7], c3072)
    LMAX = 65536
    gen = torch.Generator(device=dev)
    gen.manual_seed(55)
    dev_vecs, handles = [], []

    def P(t):
        return ctypes.c_void_p(t.data_ptr())

    server = hg.Server(ctx, budget_bytes=40 << 30, slots=args.slots, max_batch_elems=1 << 18,
                       batch_us=args.batch_us, slice_us=args.slice_us, policy=args.policy,
                       express_us=args.express_us, express_len=args.express_len, express_share=args.express_share)
    for key in keys:
        m = torch.randint(-(2 ** 40), 2 ** 40, (LMAX,), dtype=torch.int64, device=dev, generator=gen)
        r = torch.randint(-(2 ** 31), 2 ** 31, (LMAX, key.r_limbs), dtype=torch.int32, device=dev, generator=gen)
        ct = torch.empty((LMAX, key.ct_limbs), dtype=torch.int32, device=dev)
        capi.check(lib.hg_dev_encrypt(h, key.id, P(m), P(r), P(ct), LMAX, None))
        torch.cuda.synchronize()
        dev_vecs.append(ct)
        handles.append(server.store(key, ct.cpu().numpy().view(np.uint32)))
    maxS, maxRL = 192, 48
    m_host = torch.randint(-(2 ** 62), 2 ** 62, (LMAX,), dtype=torch.int64).pin_memory()
    r_host = torch.randint(-(2 ** 31), 2 ** 31, (LMAX, maxRL), dtype=torch.int32).pin_memory()
    k_host = torch.randint(-(2 ** 63), 2 ** 63 - 1, (LMAX,), dtype=torch.int64).pin_memory()
    sink = torch.empty((LMAX, maxS), dtype=torch.int32).pin_memory()
    key_ids = (ctypes.c_int * len(keys))(*[k.id for k in keys])
    hnd = (ctypes.c_uint64 * len(keys))(*handles)
    weights = [0.30, 0.20, 0.25, 0.15, 0.10]  # encrypt, add, mul, sum, decrypt
    results = []
    # warm-up: a short stream
    for rate, nreq, seed in [(1000, 50, 1)] + [(rt, 0, 0) for rt in rates]:
        if nreq == 0:
            nreq = nreq_for_rate(rate)
            seed = int(rate)
        ls = capi.LoadSpec()
        ls.key_ids = ctypes.cast(key_ids, ctypes.c_void_p)
        ls.nkeys = len(keys)
        ls.handles = ctypes.cast(hnd, ctypes.c_void_p)
        ls.rate = float(rate)
        ls.nreq = nreq
        ls.len_min, ls.len_max = 1, LMAX
        for i, wv in enumerate(weights):
            ls.op_weights[i] = wv
        ls.seed = seed
        ls.m_host, ls.r_host, ls.k_host, ls.sink = (m_host.data_ptr(), r_host.data_ptr(), k_host.data_ptr(),
                                                    sink.data_ptr())
        lat = np.zeros(nreq, dtype=np.float64)
        phases = np.zeros((nreq, 3), dtype=np.float64)
        ls.phases = phases.ctypes.data
        ops = np.zeros(nreq, dtype=np.int32)
        lens = np.zeros(nreq, dtype=np.uint64)
        wall = ctypes.c_double()
        b0 = server.stats()["batches"]
        capi.check(lib.hg_probe_serve_load(server.handle, ctypes.byref(ls), ctypes.c_void_p(lat.ctypes.data),
                                           ctypes.c_void_p(ops.ctypes.data), ctypes.c_void_p(lens.ctypes.data),
                                           ctypes.byref(wall)))
        if seed == 1:
            continue
        nb = server.stats()["batches"] - b0
        offered = rate * (LMAX - 1) / np.log(LMAX)  # mean of the log-uniform length times the rate
        results.append({"rate_req_per_s": rate, "requests": nreq,
                        "offered_elems_per_s": float(offered),
                        "p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
                        "mean_ms": float(lat.mean() * 1e3),
                        "classes": _latency_classes(lat, ops, lens, 1024),
                        # short requests of encrypt / add / mul / sum: p99 of each phase (ms)
                        "short_non_decrypt_phases_p99_ms": _phase_p99(phases, ops, lens, 1024),
                        "throughput_req_per_s": nreq / wall.value,
                        "throughput_ops_per_s": float(lens.sum()) / wall.value,
                        "micro_batches": int(nb), "wall_s": wall.value})
    # the same mix through plain per-call kernels (device-resident inputs, one stream)
    rng = np.random.default_rng(99)
    mix = []
    for _ in range(300):
        ki = int(rng.integers(len(keys)))
        n = int(min(LMAX, max(1, np.floor(np.exp(rng.uniform(0, np.log(LMAX + 1)))))))
        mix.append((ki, int(rng.choice(5, p=weights)), n))
    m_d = m_host.to(dev)
    r_d = r_host.to(dev)
    k_d = k_host.to(dev)
    out_ct = torch.empty((LMAX, maxS), dtype=torch.int32, device=dev)
    out_m = torch.empty((LMAX,), dtype=torch.int64, device=dev)
    ovf = torch.empty((LMAX,), dtype=torch.uint8, device=dev)
    st = torch.cuda.Stream(device=dev)
    sp = ctypes.c_void_p(st.cuda_stream)

    def plain():
        for ki, op, n in mix:
            key, vec = keys[ki], dev_vecs[ki]
            if op == 0:
                capi.check(lib.hg_dev_encrypt(h, key.id, P(m_d), P(r_d), P(out_ct), n, sp))
            elif op == 1:
                capi.check(lib.hg_dev_add(h, key.id, P(vec), P(vec), P(out_ct), n, sp))
            elif op == 2:
                capi.check(lib.hg_dev_mul(h, key.id, P(vec), P(k_d), P(out_ct), n, sp))
            elif op == 3:
                capi.check(lib.hg_dev_sum(h, key.id, P(vec), n, P(out_ct), sp))
            else:
                capi.check(lib.hg_dev_decrypt(h, key.id, P(vec), P(out_m), P(ovf), n, sp))

    plain()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    plain()
    torch.cuda.synchronize()
    t_plain = time.perf_counter() - t0
    capi.check(lib.hg_dev_check(h))
    plain_ops = sum(n for _, _, n in mix) / t_plain
    peak_served = max(r["throughput_ops_per_s"] for r in results)
    line = {
        "metric": "Served Paillier request stream (config 5): p50/p99 latency and throughput",
        "value": peak_served, "unit": "ops/s", "n_gpus": 1, "steps": len(results), "warmup": 1,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": {"workload": "config5", "keys": "6x2048 + 2x3072 resident", "len": [1, LMAX],
                   "op_mix": dict(zip(["encrypt", "add", "mul", "sum", "decrypt"], weights)),
                   "budget_bytes": 40 << 30, "slots": args.slots, "max_batch_elems": 1 << 18,
                   "batch_us": args.batch_us or 100000.0, "slice_us": args.slice_us or 50000.0,
                   "policy": ["shortest-remaining-first", "fifo"][args.policy],
                   "express_us": args.express_us if args.express_us > 0 else None,
                   "express_len": args.express_len or None,
                   "express_share": args.express_share or None,
                   "capacity_note": "mean request = (65536-1)/ln(65536) = 5,909 elements, so rates above "
                                    "~200 req/s offer more elements/s than one GB300 serves; lower rates are "
                                    "sub-capacity"},
        "rates": results,
        "plain_per_call_ops_per_s": plain_ops,
        "served_over_plain": peak_served / plain_ops,
    }
    server.close()
    ctx.close()
    return line


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=1 << 20)
    ap.add_argument("--window", type=int, default=20)
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-parity", action="store_true", help="skip the post-timing byte comparison with paillier_z")
    ap.add_argument("--workload", choices=["config2", "config3", "config4", "config5", "ou", "wire"],
                    default="config2")
    ap.add_argument("--no-tune", action="store_true", help="skip the autotuner")
    ap.add_argument("--key-config", default=None,
                    help="explicit key config instead of the autotuner, e.g. "
                         "'variant=0,dec_variant=0,mul_window=3,dec_window=6' (profiling a fixed kernel)")
    ap.add_argument("--quick", action="store_true", help="config5: two arrival rates only")
    ap.add_argument("--batch-us", type=float, default=0.0, help="config5: server micro-batch target (0 = default)")
    ap.add_argument("--slice-us", type=float, default=0.0, help="config5: server slice per request (0 = default)")
    ap.add_argument("--slots", type=int, default=5, help="config5: concurrent micro-batches")
    ap.add_argument("--express-share", type=float, default=0.0,
                    help="config5: share of every SM's batch blocks kept for the express slots (0 = default)")
    ap.add_argument("--express-len", type=int, default=1024,
                    help="config5: requests of at most this many elements run in the latency class (0 = off)")
    ap.add_argument("--no-extras", action="store_true",
                    help="default workload: skip the reductions, batched and served summaries")
    ap.add_argument("--policy", type=int, default=0, choices=[0, 1], help="config5: 0 shortest-first, 1 fifo")
    ap.add_argument("--rates", default="", help="config5: comma-separated arrival rates (req/s)")
    ap.add_argument("--express-us", type=float, default=0.0,
                    help="config5: express-slot threshold in estimated GPU us (0 = no express slot)")
    ap.add_argument("--ops", default="encrypt,add,mul,decrypt",
                    help="subset of the step's ops (for profiling one kernel)")
    args = ap.parse_args()
    args.ops = [o for o in args.ops.split(",") if o]
    if args.impl == "reference":
        return reference_arm(args)
    if args.workload == "config4":
        return c4_arm(args)
    if args.workload == "config3":
        return c3_arm(args)
    if args.workload == "config5":
        return c5_arm(args)
    if args.workload == "ou":
        return ou_arm(args)
    if args.workload == "wire":
        return wire_arm(args)
    return ours_arm(args)


if __name__ == "__main__":
    sys.exit(main())
