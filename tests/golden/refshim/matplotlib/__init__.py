"""Import sink for matplotlib (plotting is not used by the fixture script)."""
import types
import sys


class _Sink(types.ModuleType):
    def __getattr__(self, name):
        if name.startswith('__'):
            raise AttributeError(name)
        if name[:1].isupper():
            return type(name, (object,), {'__init__': lambda self, *a, **k: None})
        return _Sink(self.__name__ + '.' + name)

    def __call__(self, *a, **k):
        return _Sink('call')


for _name in ('pyplot', 'path', 'transforms', 'colors', 'cm', 'animation', 'patches', 'collections', 'ticker'):
    sys.modules['matplotlib.' + _name] = _Sink('matplotlib.' + _name)

rcParams = {}


def __getattr__(name):
    if name[:1].isupper():
        return type(name, (object,), {'__init__': lambda self, *a, **k: None})
    return _Sink('matplotlib.' + name)
