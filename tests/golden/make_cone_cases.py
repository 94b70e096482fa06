"""Writes cone_hit_cases.json: the Cone::hit known answers of the reference's
own unit test (tests/simple_test.cpp:8-101 of the jetshow project), restated
as data.  Cone: apex (0,0,0), axis +z, half-angle pi/4, big_scale 10.

  * "two":    ray (0,1,1) + t (0,1,0) -> one segment (0,-1,1) .. (0,1,1)   (:17-29)
  * "none":   24 rays, theta = j pi/8 (j<8), rr = k-1 (k<3): direction
              (2cos th, 2sin th, rr), origin (2cos(th+pi/2), 2sin(th+pi/2), rr)
              -> no intersection                                          (:31-57)
  * "apex":   8 rays, direction = origin = (cos th, sin th, 0) -> one
              degenerate segment at the apex                               (:59-80)
  * "border": 8 rays from the apex along the cone surface -> one segment
              -big_scale*d .. +big_scale*d                                 (:82-101)
Tolerance of the reference test: isMuchSmallerThan(1e-6, 1e-6), i.e. the
squared norm of the difference <= (1e-12)^2.
"""
import json
import math
import os

cases = []
cases.append({"kind": "two", "origin": [0., 1., 1.], "direction": [0., 1., 0.],
              "n": 1, "point_in": [0.0, -1.0, 1.0], "point_out": [0.0, 1.0, 1.0]})
r = 2.0
for j in range(8):
    th = j * math.pi / 8.
    for k in range(3):
        rr = k - 1.0
        cases.append({"kind": "none",
                      "direction": [r * math.cos(th), r * math.sin(th), rr],
                      "origin": [r * math.cos(th + math.pi / 2.0), r * math.sin(th + math.pi / 2.0), rr],
                      "n": 0})
for j in range(8):
    th = j * math.pi / 8.
    v = [math.cos(th), math.sin(th), 0.]
    cases.append({"kind": "apex", "direction": v, "origin": v, "n": 1, "point_in": [0., 0., 0.],
                  "point_out": [0., 0., 0.]})
for d in ([1., 0., 1.], [-1., 0., 1.], [1., 0., -1.], [-1., 0., 1.], [0., 1., 1.], [0., -1., 1.],
          [0., 1., -1.], [0., -1., -1.]):
    n = math.sqrt(d[0] ** 2 + d[1] ** 2 + d[2] ** 2)
    u = [x / n for x in d]
    cases.append({"kind": "border", "direction": d, "origin": [0., 0., 0.], "n": 1,
                  "point_in": [-10.0 * x for x in u], "point_out": [10.0 * x for x in u]})
out = {"cone": {"origin": [0., 0., 0.], "direction": [0., 0., 1.], "angle": math.pi / 4.0, "scale": 10.0},
       "tolerance_sq": 1e-24, "cases": cases}
with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "cone_hit_cases.json"), "w") as fh:
    json.dump(out, fh, indent=1)
