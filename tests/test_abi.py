"""The C-ABI library loads without a GPU and exports every declared symbol."""
import ctypes
import os
import re

import pytest

from glint_pipeline_gb300 import _abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "glint.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = set(re.findall(r"\b(glint_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_functions()
    for required in ("glint_create", "glint_step", "glint_step_device", "glint_sync", "glint_meetings",
                     "glint_destroy"):
        assert required in names, required


@pytest.mark.parametrize("name", declared_functions())
def test_symbol_exported(name):
    lib = ctypes.CDLL(_abi.library_path if os.path.exists(_abi.library_path) else _abi.load_library()._name)
    assert hasattr(lib, name), f"{name} declared in include/glint.h but not exported"


def test_struct_layouts_match_bindings():
    lib = _abi.lib()
    sizes = (ctypes.c_uint32 * 6)()
    lib.glint_struct_sizes(sizes)
    assert list(sizes) == [ctypes.sizeof(_abi.GlintConfig), ctypes.sizeof(_abi.GlintBox), 80,
                           ctypes.sizeof(_abi.GlintSchemaInit), 32, ctypes.sizeof(_abi.GlintStepStats)]


def test_defaults_follow_reference_configuration():
    lib = _abi.lib()
    c = _abi.GlintConfig()
    lib.glint_config_defaults(ctypes.byref(c), 1000)
    # util/config.h:29-41,176-178
    assert (c.grid_capacity, c.grid_amplify, c.reach_distance, c.min_meet_time, c.max_meet_time) == (50, 2.0, 2.0, 5,
                                                                                                     4096)
    assert c.num_meeting_buckets == 2000 and c.schema_update_delay == 1 and c.CTF_count == 100


def test_create_without_gpu_fails_cleanly():
    """On a machine without a GPU, creating a context reports NO_DEVICE rather
    than falling back to the CPU."""
    lib = _abi.lib()
    n = ctypes.c_int()
    cudart_count = None
    try:
        cudart = ctypes.CDLL("libcudart.so")
        cudart_count = cudart.cudaGetDeviceCount(ctypes.byref(n))
    except OSError:
        pass
    if cudart_count == 0 and n.value > 0:
        pytest.skip("a GPU is visible")
    import numpy as np
    from glint_pipeline_gb300 import Configuration, DeviceBench, GlintError
    pts = np.zeros((100, 2))
    with pytest.raises(GlintError) as ei:
        DeviceBench(Configuration(num_objects=100), [0, 0, 1, 1], pts)
    assert ei.value.status in (7, 2)
