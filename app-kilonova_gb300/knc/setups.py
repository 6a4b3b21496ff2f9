"""Reader of the reference's setup files (setups/*.yaml schema).

`Configuration { hydro, model, mesh, control }` (src/app.rs:167-172): `hydro`
and `model` are externally tagged enums with snake_case tags
(`relativistic` / `newtonian`, src/app.rs:68-89), every struct denies
unknown fields. The image has no YAML library, so this module parses the
subset those files use: nested block mappings by indentation, scalars
(numbers in any float spelling, booleans, `~` / `null`, bare or quoted
strings) and `#` comments.
"""
from __future__ import annotations

import re
from dataclasses import dataclass
from pathlib import Path

from .config import (SETUP_MODELS, ConfigError, Control, Mesh, NewtonianHydro, RelativisticHydro)

_NUM = re.compile(r"^[+-]?(\d+\.?\d*|\.\d+)([eE][+-]?\d+)?$")


def _scalar(s: str):
    s = s.strip()
    if s in ("~", "null", "Null", "NULL", ""):
        return None
    if s in ("true", "True", "TRUE"):
        return True
    if s in ("false", "False", "FALSE"):
        return False
    if len(s) >= 2 and s[0] == s[-1] and s[0] in "'\"":
        return s[1:-1]
    if _NUM.match(s):
        if re.match(r"^[+-]?\d+$", s):
            return int(s)
        return float(s)
    return s


def _strip_comment(line: str) -> str:
    out, quote = [], None
    for ch in line:
        if quote:
            if ch == quote:
                quote = None
        elif ch in "'\"":
            quote = ch
        elif ch == "#":
            break
        out.append(ch)
    return "".join(out).rstrip()


def parse_yaml(text: str) -> dict:
    """Parse the block-mapping subset of YAML into nested dicts."""
    root: dict = {}
    stack = [(-1, root)]
    for lineno, raw in enumerate(text.splitlines(), 1):
        line = _strip_comment(raw)
        if not line.strip():
            continue
        if "\t" in line[: len(line) - len(line.lstrip())]:
            raise ConfigError(f"line {lineno}: tabs are not allowed in indentation")
        indent = len(line) - len(line.lstrip(" "))
        body = line.strip()
        if ":" not in body:
            raise ConfigError(f"line {lineno}: expected 'key: value'")
        key, _, value = body.partition(":")
        key = key.strip()
        while stack and indent <= stack[-1][0]:
            stack.pop()
        if not stack:
            raise ConfigError(f"line {lineno}: bad indentation")
        parent = stack[-1][1]
        if key in parent:
            raise ConfigError(f"line {lineno}: duplicate key '{key}'")
        if value.strip() == "":
            child: dict = {}
            parent[key] = child
            stack.append((indent, child))
        else:
            parent[key] = _scalar(value)
    return root


@dataclass
class Configuration:
    hydro: object
    model_name: str
    model_params: dict
    mesh: Mesh
    control: Control

    def device_model(self):
        """The device model of this setup, or None when only a host callback
        can evaluate it (halo_kilonova, wind_shock). Unknown fields raise, as
        the reference's deny_unknown_fields does."""
        cls = SETUP_MODELS.get(self.model_name)
        if cls is None:
            return None
        names = {f for f in cls.__dataclass_fields__}
        extra = set(self.model_params) - names
        if extra:
            raise ConfigError(f"unknown field(s) {sorted(extra)} for {self.model_name}")
        return cls(**self.model_params)


def _one_tag(d, what):
    if not isinstance(d, dict) or len(d) != 1:
        raise ConfigError(f"{what} must be a single tagged entry")
    return next(iter(d.items()))


def load_setup(source) -> Configuration:
    """Configuration from YAML text or a path to a setups/*.yaml file."""
    text = Path(source).read_text() if (isinstance(source, Path) or
                                       (isinstance(source, str) and source.endswith(".yaml"))) else source
    d = parse_yaml(text)
    extra = set(d) - {"hydro", "model", "mesh", "control"}
    if extra:
        raise ConfigError(f"unknown field(s) {sorted(extra)} for Configuration")
    for k in ("hydro", "model", "mesh", "control"):
        if k not in d:
            raise ConfigError(f"missing field '{k}'")
    tag, hp = _one_tag(d["hydro"], "hydro")
    if tag == "relativistic":
        hydro = RelativisticHydro.from_dict(hp)
    elif tag == "newtonian":
        hydro = NewtonianHydro.from_dict(hp)
    else:
        raise ConfigError(f"unknown hydro '{tag}'")
    hydro.validate()
    model_name, model_params = _one_tag(d["model"], "model")
    mesh = Mesh.from_dict(d["mesh"])
    control = Control.from_dict(d["control"])
    mesh.validate(control.start_time)
    return Configuration(hydro, model_name, dict(model_params or {}), mesh, control)
