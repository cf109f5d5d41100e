"""xxhash stand-in built on blake2b; only the grid-cache keys change."""
import hashlib


class xxh64(object):
    def __init__(self, data=b'', seed=0):
        self._h = hashlib.blake2b(digest_size=8)
        if data:
            self.update(data)

    def update(self, data):
        self._h.update(bytes(memoryview(data)))

    def intdigest(self):
        return int.from_bytes(self._h.digest(), 'little')

    def hexdigest(self):
        return self._h.hexdigest()

    def digest(self):
        return self._h.digest()


def xxh64_intdigest(data, seed=0):
    return xxh64(data, seed).intdigest()


def xxh64_hexdigest(data, seed=0):
    return xxh64(data, seed).hexdigest()
