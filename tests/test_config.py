"""emc.conf reading (configs.cpp:40-90 keys, libconfig syntax subset)."""
import os

import pytest

import emc_gb300 as E

CONF = """
# a configuration in the reference's format
model_side = 128; #64
read_stride = 2;
wavelength = 1.03e-9;
pixel_size = 75.0e-6;
detector_size = 1024;
detector_distance = 740.0e-3;
rotations_n = 8;
sigma_start = 0.4;
sigma_final = 0.12;
sigma_half_life = 25;
diff_type = "poisson";
slice_chunk = 5000;
N_images = 20000;
max_iterations = 30; /* block
   comment */
image_prefix = "/data/" "patterns_";
mask_file = "/data/mask.bin";
normalize_images = true;
known_intensity = FALSE;
model_input = 0;
output_period = 1; output_loop = 0;
isOutput = 1
isDebug = 0;
nGPU : 1;
"""


def test_parses_every_key(built):
    c = E.read_config(text=CONF)
    assert (c.model_side, c.read_stride, c.rotations_n, c.N_images, c.max_iterations) == (
        128, 2, 8, 20000, 30)
    assert c.wavelength == 1.03e-9 and c.pixel_size == 75e-6 and c.detector_distance == 0.74
    assert c.sigma_start == 0.4 and c.sigma_final == 0.12 and c.sigma_half_life == 25
    assert c.diff == E.DIFF_POISSON
    assert c.image_prefix == b"/data/patterns_" and c.mask_file == b"/data/mask.bin"
    assert c.normalize_images == 1 and c.known_intensity == 0 and c.model_input == 0
    assert c.isOutput == 1 and c.isDebug == 0 and c.nGPUs == 1 and c.output_period == 1


def test_defaults_for_missing_keys(built):
    c = E.read_config(text="model_side = 32; N_images = 10;")
    assert c.model_side == 32 and c.rotations_n == 12 and c.nGPUs == 1
    assert c.blur_image == 0 and c.model_blur == 0.0 and c.exclude_ratio == 0.0


@pytest.mark.parametrize("bad", ["model_side 64;", "model_side = ;", 'diff_type = "fancy";',
                                 "model_side = \"x\";", "N_images = 0;", 'mask_file = "open'])
def test_errors_are_reported(built, bad):
    with pytest.raises(E.EmcError, match="config"):
        E.read_config(text=bad)


def test_diff_types(built):
    for s, d in (("absolute", E.DIFF_ABSOLUTE), ("poisson", E.DIFF_POISSON),
                 ("relative", E.DIFF_RELATIVE), ("true_poisson", E.DIFF_TRUE_POISSON)):
        assert E.read_config(text=f'diff_type = "{s}";').diff == d


def test_reference_emc_conf_if_present(built):
    from oracle.build import ref_dir
    ref = ref_dir()
    path = os.path.join(str(ref), "emc.conf") if ref else ""
    if not path or not os.path.exists(path):
        pytest.skip("reference tree not present")
    c = E.read_config(path)
    assert c.model_side == 64 and c.rotations_n == 12 and c.diff == E.DIFF_POISSON
    assert c.model_input == 2 and c.isDebug == 4 and c.normalize_images == 1


def test_missing_file(built, tmp_path):
    with pytest.raises(E.EmcError, match="cannot open"):
        E.read_config(tmp_path / "nope.conf")
