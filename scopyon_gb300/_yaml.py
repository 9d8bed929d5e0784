"""A small YAML loader for scopyon configuration files.

The configuration trees that scopyon reads (its packaged ``scopyon.yaml`` and the
strings passed to ``Configuration.update``, reference ``src/scopyon/config.py:67-78``)
use a narrow part of YAML: block mappings nested by indentation, scalars, flow
sequences such as ``[!!int 512, !!int 512]``, block sequences of scalars, the
``!!int`` / ``!!float`` / ``!!bool`` / ``!!str`` tags, quoted strings and ``#``
comments.  PyYAML is not a dependency of this package, so that subset is parsed
here.  Anything outside it raises ``ValueError`` with the offending line number.
"""

import re

__all__ = ["load"]

_INT_RE = re.compile(r"^[-+]?(0|[1-9][0-9_]*)$")
_FLOAT_RE = re.compile(r"^[-+]?(\d[\d_]*\.?\d*([eE][-+]?\d+)?|\.\d+([eE][-+]?\d+)?)$")
_SPECIAL_FLOATS = {".inf": float("inf"), "+.inf": float("inf"), "-.inf": float("-inf"),
                   ".nan": float("nan"), ".Inf": float("inf"), "-.Inf": float("-inf"),
                   ".NaN": float("nan")}


def _strip_comment(line):
    """Remove a trailing ``#`` comment that is outside quotes."""
    out = []
    quote = None
    for i, ch in enumerate(line):
        if quote:
            out.append(ch)
            if ch == quote:
                quote = None
        elif ch in "\"'":
            quote = ch
            out.append(ch)
        elif ch == "#" and (i == 0 or line[i - 1] in " \t"):
            break
        else:
            out.append(ch)
    return "".join(out).rstrip()


def _scalar(text, lineno):
    text = text.strip()
    tag = None
    if text.startswith("!!"):
        parts = text.split(None, 1)
        tag = parts[0][2:]
        text = parts[1] if len(parts) > 1 else ""
    if len(text) >= 2 and text[0] == text[-1] and text[0] in "\"'":
        value = text[1:-1]
        if text[0] == '"':
            value = value.encode("utf-8").decode("unicode_escape")
        return _apply_tag(value, tag, lineno)
    if text.startswith("["):
        if not text.endswith("]"):
            raise ValueError("line %d: unterminated flow sequence" % lineno)
        inner = text[1:-1].strip()
        if not inner:
            return []
        return [_scalar(item, lineno) for item in _split_flow(inner, lineno)]
    if text.startswith("{"):
        if not text.endswith("}"):
            raise ValueError("line %d: unterminated flow mapping" % lineno)
        inner = text[1:-1].strip()
        out = {}
        if inner:
            for item in _split_flow(inner, lineno):
                key, sep, val = item.partition(":")
                if not sep:
                    raise ValueError("line %d: bad flow mapping item %r" % (lineno, item))
                out[_scalar(key, lineno)] = _scalar(val, lineno)
        return out
    return _apply_tag(_plain(text), tag, lineno)


def _split_flow(inner, lineno):
    items, depth, quote, cur = [], 0, None, []
    for ch in inner:
        if quote:
            cur.append(ch)
            if ch == quote:
                quote = None
            continue
        if ch in "\"'":
            quote = ch
        elif ch in "[{":
            depth += 1
        elif ch in "]}":
            depth -= 1
        elif ch == "," and depth == 0:
            items.append("".join(cur))
            cur = []
            continue
        cur.append(ch)
    if quote or depth:
        raise ValueError("line %d: unbalanced flow collection" % lineno)
    items.append("".join(cur))
    return [item for item in items if item.strip()]


def _plain(text):
    if text in ("", "~", "null", "Null", "NULL"):
        return None
    if text in ("true", "True", "TRUE", "yes", "Yes", "on", "On"):
        return True
    if text in ("false", "False", "FALSE", "no", "No", "off", "Off"):
        return False
    if _INT_RE.match(text):
        return int(text.replace("_", ""))
    if text in _SPECIAL_FLOATS:
        return _SPECIAL_FLOATS[text]
    if _FLOAT_RE.match(text):
        try:
            return float(text.replace("_", ""))
        except ValueError:
            pass
    return text


def _apply_tag(value, tag, lineno):
    if tag is None:
        return value
    if tag == "int":
        return int(value)
    if tag == "float":
        return float(value)
    if tag == "bool":
        if isinstance(value, bool):
            return value
        raise ValueError("line %d: !!bool wants true/false, got %r" % (lineno, value))
    if tag == "str":
        return str(value)
    raise ValueError("line %d: unsupported tag !!%s" % (lineno, tag))


def load(text):
    """Parse ``text`` and return the nested dict / list / scalar it describes."""
    lines = []
    for lineno, raw in enumerate(text.splitlines(), start=1):
        if raw.strip() in ("---", "..."):
            continue
        if "\t" in raw[: len(raw) - len(raw.lstrip())]:
            raise ValueError("line %d: tabs are not allowed for indentation" % lineno)
        stripped = _strip_comment(raw)
        if stripped.strip():
            lines.append((len(stripped) - len(stripped.lstrip(" ")), stripped.strip(), lineno))
    if not lines:
        return None
    value, pos = _parse_block(lines, 0, lines[0][0])
    if pos != len(lines):
        raise ValueError("line %d: unexpected indentation" % lines[pos][2])
    return value


def _parse_block(lines, pos, indent):
    if lines[pos][1].startswith("- ") or lines[pos][1] == "-":
        return _parse_seq(lines, pos, indent)
    return _parse_map(lines, pos, indent)


def _parse_seq(lines, pos, indent):
    out = []
    while pos < len(lines) and lines[pos][0] == indent and (
            lines[pos][1].startswith("- ") or lines[pos][1] == "-"):
        _, text, lineno = lines[pos]
        item = text[1:].strip()
        pos += 1
        if item:
            out.append(_scalar(item, lineno))
        elif pos < len(lines) and lines[pos][0] > indent:
            value, pos = _parse_block(lines, pos, lines[pos][0])
            out.append(value)
        else:
            out.append(None)
    return out, pos


def _parse_map(lines, pos, indent):
    out = {}
    while pos < len(lines) and lines[pos][0] == indent:
        _, text, lineno = lines[pos]
        key, value_text = _split_key(text, lineno)
        pos += 1
        if value_text:
            out[key] = _scalar(value_text, lineno)
        elif pos < len(lines) and lines[pos][0] > indent:
            out[key], pos = _parse_block(lines, pos, lines[pos][0])
        elif (pos < len(lines) and lines[pos][0] == indent
              and (lines[pos][1].startswith("- ") or lines[pos][1] == "-")):
            out[key], pos = _parse_seq(lines, pos, indent)
        else:
            out[key] = None
    if pos < len(lines) and lines[pos][0] > indent:
        raise ValueError("line %d: unexpected indentation" % lines[pos][2])
    return out, pos


def _split_key(text, lineno):
    quote = None
    for i, ch in enumerate(text):
        if quote:
            if ch == quote:
                quote = None
            continue
        if ch in "\"'":
            quote = ch
        elif ch == ":" and (i + 1 == len(text) or text[i + 1] == " "):
            key = text[:i].strip()
            if len(key) >= 2 and key[0] == key[-1] and key[0] in "\"'":
                key = key[1:-1]
            return key, text[i + 1:].strip()
    raise ValueError("line %d: expected 'key: value', got %r" % (lineno, text))
