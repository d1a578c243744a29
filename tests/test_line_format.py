"""The printed line list, byte for byte: gi_format_line_text (the formatter
gi_format_lines uses) against golden text made by the reference's own printf
sequence (cuda_host.cu:1444-1473) on the same field values
(tests/golden/make_line_format.py).  Host code only."""
import json
import os

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def cases():
    return json.load(open(os.path.join(HERE, "golden", "line_format_ref.json")))


@pytest.mark.parametrize("k", range(4))
def test_line_text_matches_reference_printf(pkg, k):
    c = cases()[k]
    assert pkg.format_line_text(c["fields"]) == c["text"]


def test_line_text_rejects_bad_fields(pkg):
    f = dict(cases()[0]["fields"])
    f["ndegF"] = 3
    with pytest.raises(pkg.GiError):
        pkg.format_line_text(f)
