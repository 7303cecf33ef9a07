"""Render a few waves of a generated scene, the last one inside an NVTX range, for profilers.

``python -m crystal2_gb300.profile_wave --scene slit_room --res 480x270 --integrator guided``
renders ``--waves`` waves of ``--spp-per-wave`` samples (the guided integrator trains on them),
then one more wave between ``nvtx.range_push(--range)`` and ``range_pop``, so that a profiler can
restrict its capture to that wave (``ncu --nvtx --nvtx-include "<range>/"``).
"""
from __future__ import annotations

import argparse
import tempfile


def main() -> int:
    import torch

    from . import Context, scenes
    from . import _native as N

    ap = argparse.ArgumentParser()
    ap.add_argument("--scene", default="slit_room", choices=["slit_room", "many_material", "cornell"])
    ap.add_argument("--res", default="480x270")
    ap.add_argument("--integrator", default="plain", choices=["plain", "guided"])
    ap.add_argument("--waves", type=int, default=6)
    ap.add_argument("--spp-per-wave", type=int, default=16)
    ap.add_argument("--guide-levels", type=int, default=2)
    ap.add_argument("--train-steps", type=int, default=4, help="Adam steps per guided wave")
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--records", type=int, default=1 << 18, help="recorded vertices per guided wave")
    ap.add_argument("--windows", type=int, default=4, help="minibatch windows per guided wave")
    ap.add_argument("--range", default="capture")
    args = ap.parse_args()
    W, H = (int(v) for v in args.res.split("x"))
    d = tempfile.mkdtemp(prefix="c2g_prof_")
    if args.scene == "slit_room":
        cp, sp = scenes.slit_room(d, width=W, height=H, spp=64, depth=12, hf_res=512)
    elif args.scene == "many_material":
        cp, sp = scenes.many_material(d, width=W, height=H, spp=64)
    else:
        cp, sp = scenes.cornell(d, width=W, height=H, spp=64)
    ctx = Context(0)
    ctx.load(cp, sp, tree=N.TREE_SAH)
    ctx.guide_config(args.lr, 0.7, 2, args.train_steps)
    ctx.guide_levels(args.guide_levels)
    ctx.guide_batch(args.records, args.windows)
    integ = N.INTEGRATOR_GUIDED if args.integrator == "guided" else N.INTEGRATOR_PATH
    slots = ((W + 7) // 8) * ((H + 7) // 8) * 64

    def wave(i: int) -> None:
        p = ctx.render_params()
        p.integrator = integ
        p.sample_begin = i * args.spp_per_wave
        p.sample_count = args.spp_per_wave
        p.wave_paths = slots * args.spp_per_wave
        ctx.render(p)

    for i in range(args.waves):
        wave(i)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push(args.range)
    wave(args.waves)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    print(f"profiled wave: {args.scene} {W}x{H} {args.integrator}, {args.spp_per_wave} spp")
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
