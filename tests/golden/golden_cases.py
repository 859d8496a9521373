"""The scenes the golden fixtures were generated from (seeded, see hwrad.scenes)."""
import os
import sys

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))),
                                "hw-radiosity_gb300"))
from hwrad import scenes  # noqa: E402

CASES = {
    # 768-triangle room: no triangle reaches area 1, so no pre-partition
    "room8": {"scene": ("room", {"q": 8})},
    # tiny room used by the smoke check
    "room4": {"scene": ("room", {"q": 4, "emitter": (0.25, 0.75)})},
    # room scaled x10: every wall triangle is split by the pre-partition up to the cap
    "bigroom": {"scene": ("room", {"q": 8, "size": 100.0}), "extra": {"-triangle": "1500"}},
    # boxes: occluders, neighbour links across box faces, split sources
    "boxes": {"scene": ("room_with_boxes", {"q": 6, "n_boxes": 4, "box_q": 1, "seed": 11, "size": 30.0}),
              "extra": {"-triangle": "2000"}},
    # several shooters per step (listCanditate's top-n)
    "room8_p3": {"scene": ("room", {"q": 8}), "extra": {"-parallel_src": "3"}},
    # the reference's float->double build
    "room8_fp64": {"scene": ("room", {"q": 8}), "fp64": True},
    # the adaptive split variant (config.h = ADAPT + ROLLBACK): the room at x6
    # scale has receivers above -adapt_area 5 that the delta-FF test splits
    "adapt_room": {"scene": ("room", {"q": 4, "size": 60.0, "emitter": (0.25, 0.75)}),
                   "extra": {"-triangle": "1500", "-converge": "10"}, "adaptive": True},
    "adapt_boxes": {"scene": ("room_with_boxes", {"q": 8, "n_boxes": 3, "box_q": 1, "seed": 5, "size": 40.0}),
                    "extra": {"-triangle": "1200", "-converge": "20"}, "adaptive": True},
}


def make_scene(case):
    kind, kw = case["scene"]
    return getattr(scenes, kind)(**kw)
