"""The build drops objects made on another architecture or with other flags
(an x86 object must never be linked on the Arm host, however new it is)."""
import os

from dgcuda_gb300 import build


def _tree(tmp_path, monkeypatch):
    b = tmp_path / "_build"
    b.mkdir()
    monkeypatch.setattr(build, "BUILD", str(b))
    monkeypatch.setattr(build, "LIB", str(tmp_path / "libdg_gb300.so"))
    monkeypatch.setattr(build, "CLI", str(tmp_path / "dgcuda"))
    for f in (b / "a.cu.o", b / "b.cpp.o", tmp_path / "libdg_gb300.so", tmp_path / "dgcuda"):
        f.write_text("x")
    return b


def test_foreign_stamp_drops_objects(tmp_path, monkeypatch):
    b = _tree(tmp_path, monkeypatch)
    (b / "STAMP").write_text("some-other-arch 0\n")
    build._check_stamp(["-O3"])
    assert not any(f.endswith(".o") for f in os.listdir(b))
    assert not (tmp_path / "libdg_gb300.so").exists() and not (tmp_path / "dgcuda").exists()
    # the new stamp is written, and a second check keeps what is then built
    (b / "c.cu.o").write_text("x")
    build._check_stamp(["-O3"])
    assert (b / "c.cu.o").exists()


def test_missing_stamp_drops_objects_and_other_flags_too(tmp_path, monkeypatch):
    b = _tree(tmp_path, monkeypatch)
    build._check_stamp(["-O3"])
    assert not (b / "a.cu.o").exists()
    (b / "d.cu.o").write_text("x")
    build._check_stamp(["-O2"])
    assert not (b / "d.cu.o").exists()
