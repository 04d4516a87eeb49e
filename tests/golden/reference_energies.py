"""The reference's own golden energies and the geometries they are quoted on.

Each entry is one assertion of the reference's test suite (apyib/tests/*.py),
total energies in hartree at the Crawford water geometry or the (H2)2 geometry
of apyib/data/molecules.py:2-10 and :46-55 (bohr, frame fixed).  The reference
asserts |E - golden| < 1e-11 for each.  Fields are zero in every case.
"""

H2O = """
O  0.000000000000  -0.143225816552   0.000000000000
H  1.638036840407   1.136548822547  -0.000000000000
H -1.638036840407   1.136548822547  -0.000000000000
symmetry c1
no_com
no_reorient
units bohr
"""

H2_2 = """
H -0.708647297046685  1.417294594093371 -0.613706561565607
H  0.                 1.417294594093371  0.613706561565607
H  0.                -1.417294594093371  0.613706561565607
H  0.708647297046686 -1.417294594093371 -0.613706561565607
no_com
no_reorient
symmetry c1
units bohr
"""

GEOMS = {"H2O": H2O, "(H2)_2": H2_2}

# (id, reference assertion, method, basis, molecule, freeze_core, E_total)
CASES = [
    ("rhf_h2o_sto3g", "apyib/tests/test_002_RHF.py:21", "RHF", "STO-3G", "H2O", False, -74.9420799281922),
    ("rhf_h2o_631gd", "apyib/tests/test_002_RHF.py:55", "RHF", "6-31G(d)", "H2O", False, -75.97474825544526),
    ("rhf_h2o_ccpvdz", "apyib/tests/test_004_CID.py:59", "RHF", "cc-pVDZ", "H2O", False, -75.98979581991861),
    ("mp2_h2o_sto3g", "apyib/tests/test_006_MP2_SO.py:21", "MP2", "STO-3G", "H2O", False, -74.9912295643122),
    ("mp2_h2o_631gd", "apyib/tests/test_006_MP2_SO.py:60", "MP2", "6-31G(d)", "H2O", False, -76.17533681889488),
    ("mp2_h2o_ccpvdz_fc", "apyib/tests/test_006_MP2_SO.py:124", "MP2", "cc-pVDZ", "H2O", True, -76.20202577979143),
    ("cid_h2o_sto3g", "apyib/tests/test_007_CID_SO.py:21", "CID", "STO-3G", "H2O", False, -75.01073817893661),
    ("cid_h2o_ccpvdz", "apyib/tests/test_007_CID_SO.py:59-60", "CID", "cc-pVDZ", "H2O", False,
     -75.98979581991861 + -0.21279410950205),
    ("cid_h2o_ccpvdz_fc", "apyib/tests/test_007_CID_SO.py:127", "CID", "cc-pVDZ", "H2O", True, -76.20078548433332),
    ("cisd_h2o_631g", "apyib/tests/test_008_CISD_SO.py:21", "CISD", "6-31G", "H2O", False, -76.09503651362023),
    ("cisd_h2o_ccpvdz", "apyib/tests/test_008_CISD_SO.py:59", "CISD", "cc-pVDZ", "H2O", False, -76.20375874728018),
    ("cisd_h22_sto3g", "apyib/tests/test_008_CISD_SO.py:122", "CISD", "STO-3G", "(H2)_2", False, -2.2165136315314133),
    ("cisd_h2o_ccpvdz_fc", "apyib/tests/test_008_CISD_SO.py:147", "CISD", "cc-pVDZ", "H2O", True, -76.20195791202802),
]

# the reference's convergence settings in these tests
PARAMS = dict(e_convergence=1e-12, d_convergence=1e-12, DIIS=True, max_iterations=120,
              F_el=[0.0, 0.0, 0.0], F_mag=[0.0, 0.0, 0.0])
