"""Minimal YAML reader, enough for the reference's default configuration file.

Only block mappings, scalars (numbers, booleans, strings, empty) and inline
lists of scalars are understood.  Used only to import the reference for fixture
generation.
"""


def _scalar(text):
    text = text.strip()
    if text == '' or text in ('~', 'null'):
        return None
    if text in ('true', 'True'):
        return True
    if text in ('false', 'False'):
        return False
    if text.startswith('[') and text.endswith(']'):
        inner = text[1:-1].strip()
        return [] if not inner else [_scalar(t) for t in inner.split(',')]
    if text[0] in '\'"' and text[-1] == text[0]:
        return text[1:-1]
    for conv in (int, float):
        try:
            return conv(text)
        except ValueError:
            pass
    return text


def safe_load(stream):
    text = stream.read() if hasattr(stream, 'read') else stream
    if isinstance(text, bytes):
        text = text.decode()
    root = {}
    stack = [(-1, root)]
    for raw in text.splitlines():
        line = raw.split('#', 1)[0].rstrip() if not raw.lstrip().startswith("'") else raw.rstrip()
        if not line.strip():
            continue
        indent = len(line) - len(line.lstrip())
        key, _, value = line.strip().partition(':')
        while stack[-1][0] >= indent:
            stack.pop()
        parent = stack[-1][1]
        if value.strip() == '':
            child = {}
            parent[key] = child
            stack.append((indent, child))
        else:
            parent[key] = _scalar(value)
    # empty mappings stand for empty values
    def fix(d):
        for k, v in d.items():
            if isinstance(v, dict):
                if not v:
                    d[k] = None
                else:
                    fix(v)
    fix(root)
    return root


load = safe_load


def safe_dump(*args, **kwargs):
    raise NotImplementedError('yaml shim cannot dump')
