"""CPU checks of the test-side HDF5 reader (tests/h5read.py) that verifies the
files iskra_write_openpmd writes: its lookup3 checksum against the values
published with Jenkins' lookup3.c (hashlittle of "" with initval 0 and
0xdeadbeef, of "Four score and seven years ago" with initval 0 and 1)."""
from h5read import lookup3


def test_lookup3_published_values():
    assert lookup3(b"") == 0xDEADBEEF
    assert lookup3(b"", 0xDEADBEEF) == 0xBD5B7DDE
    assert lookup3(b"Four score and seven years ago") == 0x17770551
    assert lookup3(b"Four score and seven years ago", 1) == 0xCD628161


def test_lookup3_block_boundaries():
    # lengths around the 12-byte block boundary take different tail paths;
    # the hash must change with every byte
    data = bytes(range(40))
    seen = {lookup3(data[:n]) for n in range(40)}
    assert len(seen) == 40
