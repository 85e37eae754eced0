"""The reference's own LM (torch, float64, CPU, one thread) against the oracle port on the same
12 stamps of 64 x 64 (own Moffat PSFs, truth perturbed by 10 %): messages, iteration counts,
chi^2 and seconds per fit side by side, to calibrate the CPU baseline (the port) against the
reference itself.  Run with ASTROPHOT_REFERENCE=<reference checkout>:

    python tests/golden/time_reference_cpu.py
"""
import os, sys, time
import numpy as np
REPO = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, REPO); sys.path.insert(0, os.path.join(REPO, "tests", "golden"))
if not os.environ.get("ASTROPHOT_REFERENCE"):
    raise SystemExit("set ASTROPHOT_REFERENCE to the reference checkout")
import torch
torch.set_num_threads(1)
import make_golden as MG
ap = MG.import_reference()
from astrophot_gb300 import synthetic
from oracle.lm import GroupProblem, LMOracle
from oracle.render import PSF, Component, Window

specs = synthetic.cutout_stamps(64, 11, lo=64, hi=64)[:12]   # 64x64 stamps, own PSFs
tr, to = [], []
for k, s in enumerate(specs):
    tgt0 = ap.image.Target_Image(data=np.zeros((64, 64)), pixelscale=1.0, psf=s.psf)
    g = MG.build_lm_group(ap, tgt0, s.truth, f"t{k}")
    truth = g().data.detach().numpy()
    data, w = synthetic.add_noise(truth, s.seed)
    tgt = ap.image.Target_Image(data=data, pixelscale=1.0, psf=s.psf, variance=1.0 / w)
    grp = MG.build_lm_group(ap, tgt, s.init, f"f{k}")
    rep0 = grp.parameters.vector_representation().detach().clone()
    t = time.perf_counter(); r = ap.fit.LM(grp, initial_state=rep0).fit(); tr.append(time.perf_counter() - t)
    cx, cy, q, PA, n, Re, Ie = s.init
    gal = Component("sersic", {"center": [cx, cy], "q": q, "PA": PA, "n": n, "Re": Re, "Ie": Ie}, psf_mode="full")
    sky = Component("flat_sky", {"F": 0.0}, locked=("F",))
    prob = GroupProblem([gal, sky], Window.from_scale(64, 64), PSF(s.psf), data, w)
    t = time.perf_counter(); o = LMOracle(prob, prob.representation()).fit(); to.append(time.perf_counter() - t)
    print(k, r.message, len(r.loss_history), o.message, len(o.loss_history), f"ref {tr[-1]:.2f}s oracle {to[-1]:.2f}s",
          f"chi2 rel {abs(min(r.loss_history)/o.res_loss()-1):.1e}", flush=True)
print("reference fits/s", len(tr) / sum(tr), "oracle fits/s", len(to) / sum(to), "ratio", sum(tr) / sum(to))
