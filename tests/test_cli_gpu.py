"""gbmm-cli (mat-gpu's command line) end to end: -i -p on the golden inputs
for every method, and -n/-b/-s random matrices against the CPU oracle."""
import subprocess

import pytest

from conftest import golden_cases, load_golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cli(built_lib):
    import build as gbuild
    return gbuild.CLI


@pytest.mark.parametrize("name", ["rect_7x13x5_zeros", "cfg1_like_16x16x16_1024b", "square_64x64x64_64b",
                                  "allones_8x8x8_256b", "tiny_1x1x1"])
@pytest.mark.parametrize("method", ["1", "3", "35", "4", "8", "0"])
def test_cli_golden(cli, name, method):
    text, expect = load_golden(name)
    out = subprocess.run([cli, "-i", "-p", "-m", method, "-B", "8"], input=text.encode(), stdout=subprocess.PIPE,
                         stderr=subprocess.PIPE, check=True)
    assert out.stdout.decode() == expect
    assert b"Time taken" in out.stderr


def test_cli_random_vs_oracle(cli, oracle):
    gen = subprocess.run([cli, "-g", "-n", "20,33,17", "-b", "777", "-s", "5"], stdout=subprocess.PIPE,
                         check=True).stdout.decode()
    exp, _ = oracle.matmul_text(gen, method=1)
    out = subprocess.run([cli, "-i", "-p", "-m", "8"], input=gen.encode(), stdout=subprocess.PIPE,
                         stderr=subprocess.DEVNULL, check=True).stdout.decode()
    assert out == exp
