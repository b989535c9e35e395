"""Plan wisdom as text (host logic, no GPU): lines of "key<TAB>value" with
22 integers per value merge by key, export sorted, and text that does not
parse is refused whole."""
import pytest

VALUE = " ".join(["1536", "0", "0"] + ["1", "128", "2", "256", "1"] * 3 +
                 ["4", "256", "4", "128"])


def _line(key, value=VALUE):
    return f"fgb1 {key}\t{value}\n"


@pytest.fixture
def wisdom(native_lib):
    from fftwpp_gb300 import gpu
    gpu.forget_wisdom()
    yield gpu
    gpu.forget_wisdom()


def test_wisdom_roundtrip_and_merge(wisdom):
    assert wisdom.export_wisdom() == ""
    assert wisdom.import_wisdom(_line("b") + _line("a")) == 2
    text = wisdom.export_wisdom()
    assert text == _line("a") + _line("b")            # sorted by key
    other = VALUE.replace("1536", "768", 1)
    assert wisdom.import_wisdom(_line("a", other)) == 1
    assert wisdom.export_wisdom() == _line("a", other) + _line("b")
    assert wisdom.import_wisdom("") == 0
    wisdom.forget_wisdom()
    assert wisdom.export_wisdom() == ""


@pytest.mark.parametrize("bad", [
    "fgb1 a 1 2 3\n",                                 # no tab
    "\t" + VALUE + "\n",                              # empty key
    "xyz a\t" + VALUE + "\n",                         # not a library key
    _line("a", VALUE + " 7"),                         # 23 numbers
    _line("a", VALUE.rsplit(" ", 1)[0]),              # 21 numbers
    _line("a", VALUE.replace("128", "-1", 1)),        # negative
    _line("a", VALUE.replace("128", "x", 1)),         # not a number
])
def test_wisdom_refuses_bad_text(wisdom, bad):
    wisdom.import_wisdom(_line("keep"))
    with pytest.raises(ValueError):
        wisdom.import_wisdom(_line("b") + bad)
    assert wisdom.export_wisdom() == _line("keep")    # nothing taken


def test_wisdom_file(wisdom, tmp_path):
    path = str(tmp_path / "wisdom.txt")
    assert wisdom.load_wisdom(path) == 0
    wisdom.import_wisdom(_line("a"))
    wisdom.save_wisdom(path)
    wisdom.forget_wisdom()
    wisdom.import_wisdom(_line("b"))
    wisdom.save_wisdom(path)                          # merges with the file
    wisdom.forget_wisdom()
    assert wisdom.load_wisdom(path) == 2
    assert wisdom.export_wisdom() == _line("a") + _line("b")
