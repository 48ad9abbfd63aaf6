"""The attribute values of the snapshot's /Header, /Cosmology and /Units groups
(writeHeaderAttributes, src/header.c:26-175), made by the library on the host; pinned against the
reference's own function.  CPU only."""
import pytest

import oracle
import mitos_gb300.lib as ml


HEADER_CASES = [
    (1000.0, 31.0, [("PartType1", 512 ** 3)], (1.98841e43, 3.08567758e22, 3.08567758e19, 1.0, 1.0)),
    (256.0, 99.5, [("PartType1", 64 ** 3), ("PartType6", 32 ** 3), ("PartType1", 7), ("Other", 5)],
     (1.0, 1.0, 1.0, 1.0, 1.0)),
    (500.0, 0.0, [], (2e30, 3e22, 3e19, 2.5, 0.5)),
]


@pytest.mark.parametrize("boxlen,z,types,units", HEADER_CASES)
def test_snapshot_header_attributes(boxlen, z, types, units):
    """every attribute writeHeaderAttributes (src/header.c:26-175) writes: the library's values
    against the reference's own function (compiled with an HDF5 stand-in that records the writes),
    or against the restated rules where the reference build is absent"""
    got = ml.snapshot_header(boxlen, z, types, units)
    ref = oracle.ref_header_attributes(boxlen, z, types, units)
    if ref is None:  # the rules of src/header.c restated
        nump = [sum(t[1] for t in types if t[0] == f"PartType{i}") for i in range(7)]
        ref = {("/Header", "BoxSize"): [boxlen] * 3, ("/Header", "Dimension"): [3], ("/Header", "Redshift"): [z],
               ("/Header", "Flag_Entropy_ICs"): [0], ("/Header", "NumFilesPerSnapshot"): [1],
               ("/Header", "NumPart_Total"): nump, ("/Header", "NumPart_Total_HighWord"): [0] * 7,
               ("/Header", "MassTable"): [0.0] * 7, ("/Cosmology", "Redshift"): [z],
               ("/Units", "Unit mass in cgs (U_M)"): [units[0] * 1000],
               ("/Units", "Unit length in cgs (U_L)"): [units[1] * 100],
               ("/Units", "Unit time in cgs (U_t)"): [units[2]],
               ("/Units", "Unit temperature in cgs (U_T)"): [units[3]],
               ("/Units", "Unit current in cgs (U_I)"): [units[4]]}
    assert set(got) == set(ref)
    for key in ref:
        assert got[key] == ref[key], key
