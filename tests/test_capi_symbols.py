"""The C-ABI library builds for sm_103a and exports every entry point that
include/*.h declares (no GPU needed: nothing is called)."""
import ctypes
import glob
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DECL = re.compile(r"^\s*(?:const\s+)?(?:int|void|char\s*\*|const\s+char\s*\*)\s*\*?\s*(fvgs_\w+)\s*\(", re.M)


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names.update(DECL.findall(src))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_symbols()
    for must in ("fvgs_session_create", "fvgs_project_bin", "fvgs_track_jacobian", "fvgs_track_frame",
                 "fvgs_map_step", "fvgs_render", "fvgs_rgbd_pose_jacobians_noalloc", "fvgs_remove_outliers",
                 "fvgs_prune", "fvgs_covisibility", "fvgs_visibility", "fvgs_init_gaussians", "fvgs_densify"):
        assert must in names


def test_library_exports_every_declared_symbol(fvgs_lib):
    lib = ctypes.CDLL(fvgs_lib.LIB_PATH)
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_status_strings_and_defaults(fvgs_lib):
    lib = fvgs_lib.load_library()
    assert lib.fvgs_status_string(0) == b"ok"
    assert lib.fvgs_status_string(-5).startswith(b"bounded")
    p = fvgs_lib.default_params()
    assert (p.tile_w, p.tile_h, p.radius_sigma) == (16, 16, 3.0)
    assert abs(p.alpha_thresh - 0.2) < 1e-7 and abs(p.color_thresh - 0.1) < 1e-7
    assert p.quirks == fvgs_lib.QUIRKS_DEFAULT
    # invalid arguments are rejected before any device work
    assert lib.fvgs_params_default(None) == -1
    assert lib.fvgs_session_create(None, 0, 0, 0, 0, None) == -1
