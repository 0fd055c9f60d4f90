"""Copy newt's own golden vectors for the stepping path into tests/golden/.

Runs only where the reference checkout is available (never on the GPU machine):
    python tests/golden/collect_fixtures.py <newt checkout>/tests
The files are byte goldens written by newt's test suite (f32 little-endian
state snapshots, newt/tests/goldens/*.bin) and MuJoCo 3.11.0 FP64 captures in
newt's NEWTDIF1 format (newt/tests/references/*.bin), plus the scene files
those captures were made from and newt's packaged JSON models
(newt/models/*.json).  They are data, copied verbatim.
"""
import os
import shutil
import sys

if len(sys.argv) != 2:
    sys.exit("usage: collect_fixtures.py <newt checkout>/tests")
REF = sys.argv[1]
OUT = os.path.dirname(os.path.abspath(__file__))

FILES = [
    "../models/stack.json",
    "../models/pendulum.json",
    "../models/arm.json",
    "../models/pile.json",
    "goldens/integrator_euler.bin",
    "goldens/integrator_rk4.bin",
    "goldens/dynamics_mass_bias.bin",
    "goldens/joints_chain_and_floating.bin",
    "goldens/solver_stack.bin",
    "goldens/solver_incline.bin",
    "goldens/solver_newton_stack.bin",
    "goldens/solver_newton_incline.bin",
    "goldens/solver_tree.bin",
    "goldens/solver_newton_tree.bin",
    "goldens/condim_torsional.bin",
    "goldens/condim_rolling.bin",
    "references/double_pendulum_euler.bin",
    "references/ballistic_euler.bin",
    "references/sphere_drop_euler.bin",
    "references/sphere_drop_newton_euler.bin",
    "references/box_stack_euler.bin",
    "references/box_stack_newton_euler.bin",
    "references/tree_chain_contact_newton_euler.bin",
    "references/tree_chain_contact_pgs_euler.bin",
    "references/box_plane_mujoco_anchors.json",
    "references/ballistic.xml",
    "references/sphere_drop.xml",
    "references/sphere_drop_stiff.xml",
    "references/sphere_drop_soft.xml",
    "references/sphere_drop_stiff_euler.bin",
    "references/sphere_drop_soft_euler.bin",
    "references/box_stack.xml",
    "references/double_pendulum.xml",
    "references/tree_chain_contact.xml",
    "references/constraint_factor_diagnostics.json",
]

for rel in FILES:
    src = os.path.join(REF, rel)
    dst = os.path.join(OUT, os.path.basename(rel))
    shutil.copyfile(src, dst)
    print(f"{rel} -> {os.path.relpath(dst)} ({os.path.getsize(dst)} bytes)")
