"""Failure paths, made on the host: no GPU fault, trap or hang is provoked.

SKY_FAULT is read once per process, so each case runs in a child process:

* lookback:N -- the N-th radix sort of the process runs its bounded
  look-back waits out (tile 0 withholds its look-back word and the waits
  give up after 64 polls).  The call must return SKY_ERR_TIMEOUT, change no
  parameter, and the next call on the same context or the same device
  pointers must succeed with the correct result.  (The reference's
  look-back, radix_sort.wgsl:372-393, has no bound.)
* alloc:N -- the N-th device allocation fails: SKY_ERR_INJECTED, and a
  retry of the same call succeeds with the same device memory as a context
  that never failed (nothing leaked or counted twice).
* launch:N -- the N-th pass fails before it launches anything: parameters
  and counters unchanged, and the next step equals a clean first step.
"""
import json
import os
import subprocess
import sys
import textwrap

import pytest

from conftest import PKG, REPO

pytestmark = pytest.mark.gpu

PRELUDE = f"""
import sys, json, ctypes as C
sys.path[:0] = [{str(REPO)!r}, {str(PKG)!r}]
import numpy as np
import skyfall as sky
from skyfall import scenes
L = sky.lib()
E = sky._lib

def scene():
    P = scenes.scene_clusters(20000, seed=1901, clusters=16, center_range=1.0,
                              cluster_sigma=0.25, logscale_mean=-3.8)
    cams = scenes.cameras_orbit(2, 3.5, 320, 240)
    tgts = [scenes.target_uniform(320, 240, seed=2900 + k) for k in range(2)]
    return P, cams, tgts

def make(P, cams, tgts, **kw):
    r = sky.GaussianRenderer(sh_degree=3, sh_degree_interval=0, w_l2=1.0, w_l1=0.2,
                             w_ssim=0.0, **kw)
    r.load_points(P)
    r.setTrainingCameras(cams)
    r.setTrainingImages(tgts)
    return r

def rc_of(fn, *a):
    try:
        fn(*a)
        return 0
    except E.SkyError as e:
        return e.code
"""


def run_child(fault: str, body: str) -> dict:
    env = dict(os.environ, SKY_FAULT=fault)
    code = PRELUDE + textwrap.dedent(body)
    p = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True,
                       timeout=600)
    assert p.returncode == 0, p.stdout + p.stderr
    return json.loads(p.stdout.strip().splitlines()[-1])


def test_sort_lookback_timeout_is_reported_and_the_next_sort_is_correct(sky):
    out = run_child("lookback:1", """
        import torch
        rng = np.random.default_rng(5)
        keys = rng.integers(0, 2**32, 200_000, dtype=np.uint64).astype(np.uint32)
        kin = torch.from_numpy(keys.view(np.int32)).cuda()
        kout = torch.empty_like(kin); vout = torch.empty_like(kin)
        st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        p = lambda t: C.c_void_p(t.data_ptr())
        rc1 = L.sky_sort_pairs(p(kin), None, p(kout), p(vout), keys.size, 32, st)
        msg = L.sky_last_error().decode()
        rc2 = L.sky_sort_pairs(p(kin), None, p(kout), p(vout), keys.size, 32, st)
        torch.cuda.synchronize()
        order = np.argsort(keys, kind="stable")
        ok = bool(np.array_equal(kout.cpu().numpy().view(np.uint32), keys[order]) and
                  np.array_equal(vout.cpu().numpy().view(np.uint32), order.astype(np.uint32)))
        print(json.dumps(dict(rc1=rc1, msg=msg, rc2=rc2, ok=ok)))
    """)
    assert out["rc1"] == sky._lib.SKY_ERR_TIMEOUT
    assert "look-back" in out["msg"]
    assert out["rc2"] == 0 and out["ok"]


def test_step_with_timed_out_sort_changes_nothing_and_the_next_step_is_clean(sky):
    out = run_child("lookback:1", """
        P, cams, tgts = scene()
        r = make(P, cams, tgts)            # direct launches: the first sort of the step fails
        p0 = r.params()
        rc1 = rc_of(r.trainStep, [0, 1])
        st = r.getStatus()
        unchanged = bool(np.array_equal(r.params().view(np.uint32), p0.view(np.uint32)))
        s2 = r.trainStep([0, 1])
        clean = make(P, cams, tgts)
        s3 = clean.trainStep([0, 1])
        same = bool(np.array_equal(r.params().view(np.uint32), clean.params().view(np.uint32)))
        print(json.dumps(dict(rc1=rc1, it_after_fail=int(st.iteration), flags=int(st.error_flags),
                              unchanged=unchanged, it2=int(s2.iteration), loss2=s2.loss,
                              loss3=s3.loss, same=same)))
    """)
    assert out["rc1"] == sky._lib.SKY_ERR_TIMEOUT
    assert out["it_after_fail"] == 0 and out["unchanged"]
    assert out["flags"] & 2  # the sticky device error word records the timeout
    assert out["it2"] == 1 and out["loss2"] == out["loss3"] and out["same"]


def test_graph_step_after_a_timed_out_direct_step(sky):
    """The first step runs directly (it sizes the buffers); it times out.
    The graph-captured steps after it are clean and equal a clean context's."""
    out = run_child("lookback:2", """
        P, cams, tgts = scene()
        r = make(P, cams, tgts, use_graph=1)
        rc1 = rc_of(r.trainStep, [0, 1])   # sorts: item sort (1), intersection sort (2)
        losses = [r.trainStep([0, 1]).loss for _ in range(3)]
        clean = make(P, cams, tgts, use_graph=1)
        ref = [clean.trainStep([0, 1]).loss for _ in range(3)]
        same = bool(np.array_equal(r.params().view(np.uint32), clean.params().view(np.uint32)))
        print(json.dumps(dict(rc1=rc1, losses=losses, ref=ref, same=same,
                              replays=int(r.getStatus().graph_replays))))
    """)
    assert out["rc1"] == sky._lib.SKY_ERR_TIMEOUT
    assert out["losses"] == out["ref"] and out["same"]
    assert out["replays"] >= 2


def test_injected_allocation_failure_then_clean_retry(sky):
    # allocation 12 falls inside the first training step's buffer set-up
    out = run_child("alloc:12", """
        P, cams, tgts = scene()
        r = make(P, cams, tgts)
        p0 = r.params()
        rc1 = rc_of(r.trainStep, [0, 1])
        msg = L.sky_last_error().decode()
        unchanged = bool(np.array_equal(r.params().view(np.uint32), p0.view(np.uint32)))
        s2 = r.trainStep([0, 1])
        b_retry = int(r.getStatus().device_bytes)
        clean = make(P, cams, tgts)
        s3 = clean.trainStep([0, 1])
        print(json.dumps(dict(rc1=rc1, msg=msg, unchanged=unchanged, loss2=s2.loss, loss3=s3.loss,
                              b_retry=b_retry, b_clean=int(clean.getStatus().device_bytes))))
    """)
    assert out["rc1"] == sky._lib.SKY_ERR_INJECTED and "injected" in out["msg"]
    assert out["unchanged"]
    assert out["loss2"] == out["loss3"]
    assert out["b_retry"] == out["b_clean"]


def test_injected_launch_failure_changes_nothing(sky):
    out = run_child("launch:1", """
        P, cams, tgts = scene()
        r = make(P, cams, tgts)
        p0 = r.params()
        rc1 = rc_of(r.trainStep, [0, 1])
        st = r.getStatus()
        unchanged = bool(np.array_equal(r.params().view(np.uint32), p0.view(np.uint32)))
        s2 = r.trainStep([0, 1])
        clean = make(P, cams, tgts)
        s3 = clean.trainStep([0, 1])
        same = bool(np.array_equal(r.params().view(np.uint32), clean.params().view(np.uint32)))
        print(json.dumps(dict(rc1=rc1, it=int(st.iteration), launches=int(st.kernel_launches),
                              unchanged=unchanged, loss2=s2.loss, loss3=s3.loss, same=same)))
    """)
    assert out["rc1"] == sky._lib.SKY_ERR_INJECTED
    assert out["it"] == 0 and out["launches"] == 0 and out["unchanged"]
    assert out["loss2"] == out["loss3"] and out["same"]
