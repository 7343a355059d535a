"""oxRNA2 model: RNA geometry and constants over the same force engine.

Same public names, constants and signatures as the reference's
``oxdna/model/rna2.py`` (constants of oxDNA's ``rna_model.h``). The RNA forms of
stacking (asymmetric STACK_3/STACK_5 sites, backbone angles), cross-stacking
(theta4 dropped) and coaxial stacking (two dihedrals from the real BACK vector) are
selected by parameters.
"""

import itertools
import math

from .. import runtime
from ..forces import (CoaxialStacking, CrossStacking, DebyeHuckel, ExcludedVolume,
                      HydrogenBonding, OxDNABonded)
from ..io import DNA_BASES
from . import dna1

POS_BASE = 0.40
POS_STACK = 0.34
BACK_SITE = (-0.40, 0.0, 0.20)
BASE_SITE = (POS_BASE, 0.0, 0.0)
STACK_SITE = (POS_STACK, 0.0, 0.0)

FENE_EPS = 2.0
FENE_R0 = 0.761070781051
FENE_DELTA = 0.25

EXCL_EPS = 2.0
EXCL = dna1.EXCL
EXCVOL_R_CUT = 2.0

HYDR_EPS = 0.870439
HYDR_A, HYDR_RC, HYDR_R0 = 8.0, 0.75, 0.4
HYDR_RLOW, HYDR_RHIGH, HYDR_RCLOW, HYDR_RCHIGH = 0.34, 0.7, 0.276908, 0.783775
HYDR_BLOW, HYDR_BHIGH = -126.243, -7.87708
HB_F4_THETA1 = (1.5, 4.16038, 0.0, 0.7, 0.952381)
HB_F4_THETA23 = (1.5, 4.16038, 0.0, 0.7, 0.952381)
HB_F4_THETA4 = (0.46, 0.133855, math.pi, 0.7, 3.10559)
HB_F4_THETA78 = (4.0, 17.0526, math.pi / 2.0, 0.45, 0.555556)
HB_R_CUT = HYDR_RCHIGH + 2.0 * POS_BASE

ST_T_DEP = 1.97561
STCK_SEQ = {
    ("G", "C"): 1.27562, ("C", "G"): 1.60302, ("G", "G"): 1.49422, ("C", "C"): 1.47301,
    ("G", "A"): 1.62114, ("T", "C"): 1.16724, ("A", "G"): 1.39374, ("C", "T"): 1.47145,
    ("T", "G"): 1.28576, ("C", "A"): 1.58294, ("G", "T"): 1.57119, ("A", "C"): 1.21041,
    ("A", "T"): 1.38529, ("T", "A"): 1.24573, ("A", "A"): 1.31585, ("T", "T"): 1.17518,
}
HYDR_SEQ = {("A", "T"): 0.820419, ("T", "A"): 0.820419, ("C", "G"): 1.06444,
            ("G", "C"): 1.06444, ("G", "T"): 0.510558, ("T", "G"): 0.510558}

CRST_F2 = (59.9626, 0.5, 0.6, 0.42, 0.58, 0.375, 0.625, -0.888889, -0.888889)
CRST_F4_THETA1 = (2.25, 7.00545, 0.505, 0.58, 0.766284)
CRST_F4_THETA23 = (1.70, 6.2469, 1.266, 0.68, 0.865052)
CRST_F4_THETA4 = (1.50, 2.59556, 0.0, 0.65, 1.02564)
CRST_F4_THETA78 = (1.70, 6.2469, 0.309, 0.68, 0.865052)
CRST_RCHIGH = 0.625
CROSS_R_CUT = CRST_RCHIGH + 2.0 * POS_BASE

CXST_F2 = (80.0, 0.5, 0.6, 0.42, 0.58, 0.375, 0.625, -0.888889, -0.888889)
CXST_F4_THETA1 = (2.0, 10.9032, 2.592, 0.65, 0.769231)
CXST_F4_THETA4 = (1.3, 6.4381, 0.151, 0.8, 0.961538)
CXST_F4_THETA56 = (0.9, 3.89361, 0.685, 0.95, 1.16959)
CXST_F5_PHI3 = (2.0, 10.9032, -0.769231, -0.65)
CXST_F5_PHI4 = (2.0, 10.9032, -0.769231, -0.65)
CXST_RCHIGH = 0.625
COAX_R_CUT = CXST_RCHIGH + 2.0 * POS_STACK

DH_LAMBDA_FACTOR = 0.3667258
DH_PREFACTOR = 0.0858
DEFAULT_SALT = 1.0

STACK_3_SITE = (0.4, 0.1, 0.0)
STACK_5_SITE = (0.124906078525, -0.00866274917473, 0.0)
BBVECTOR_3 = (-0.462510, -0.528218, 0.712089)
BBVECTOR_5 = (-0.104402, -0.841783, 0.529624)
STCK_BASE_EPS = 1.40206
STCK_FACT_EPS = 2.77
STCK_A, STCK_RC, STCK_R0 = 6.0, 0.93, 0.43
STCK_RLOW, STCK_RHIGH, STCK_RCLOW, STCK_RCHIGH = 0.35, 0.78, 0.26239, 0.986
STCK_BLOW, STCK_BHIGH = -68.1857, -3.12992
STCK_F4_THETA5 = (0.9, 3.89361, 0.0, 0.95, 1.16959)
STCK_F4_THETAB1 = (1.3, 6.4381, 0.0, 0.8, 0.961538)
STCK_F4_THETAB2 = (1.3, 6.4381, 0.0, 0.8, 0.961538)
STCK_F5_PHI1 = (2.0, 10.9032, -0.769231, -0.65)


def _all_pairs(types):
    return itertools.combinations_with_replacement(types, 2)


def cross_stacking(nlist, types=DNA_BASES, r_cut=CROSS_R_CUT):
    """oxRNA2 cross-stacking: theta4 factor dropped (t4_enabled=False)."""
    force = CrossStacking(nlist=nlist, default_r_cut=r_cut, mode="none")
    pair = dict(base_site=BASE_SITE, f2=CRST_F2, f4_t1=CRST_F4_THETA1, f4_t23=CRST_F4_THETA23,
                f4_t4=CRST_F4_THETA4, f4_t78=CRST_F4_THETA78, t4_enabled=False)
    for a, b in _all_pairs(types):
        force.params[(a, b)] = dict(pair)
    return force


def coaxial_stacking(nlist, types=DNA_BASES, r_cut=COAX_R_CUT):
    """oxRNA2 coaxial stacking (two dihedrals from the real BACK-BACK vector)."""
    force = CoaxialStacking(nlist=nlist, default_r_cut=r_cut, mode="none")
    pair = dict(stack_site=STACK_SITE, stack_back_ref=BACK_SITE, gamma=0.0, f2=CXST_F2,
                f4_t1=CXST_F4_THETA1, f4_t4=CXST_F4_THETA4, f4_t56=CXST_F4_THETA56,
                f5_phi3=CXST_F5_PHI3, f5_phi4=CXST_F5_PHI4, t1_mode=0, t1_sa=0.0, t1_sb=0.0,
                phi3_enabled=False, rna_coax=True)
    for a, b in _all_pairs(types):
        force.params[(a, b)] = dict(pair)
    return force


def sequence_stacking_eps_table(t_kelvin=296.15):
    factor = 1.0 + dna1.kT_from_temperature(t_kelvin) * ST_T_DEP
    return [[STCK_SEQ[(a, b)] * factor for b in DNA_BASES] for a in DNA_BASES]


def stacking_params(t_kelvin=296.15, average=True):
    shift = (1.0 - math.exp(-(STCK_RC - STCK_R0) * STCK_A)) ** 2
    f1 = (STCK_A, STCK_R0, STCK_RLOW, STCK_RHIGH, STCK_RCLOW, STCK_RCHIGH, STCK_BLOW,
          STCK_BHIGH, shift)
    if average:
        eps_flat = (STCK_BASE_EPS + STCK_FACT_EPS * dna1.kT_from_temperature(t_kelvin),) * 16
    else:
        t = sequence_stacking_eps_table(t_kelvin)
        eps_flat = tuple(t[i][j] for i in range(4) for j in range(4))
    return dict(stack_enabled=True, stack_rna=True, stack_f1=f1, stack_eps=eps_flat,
                stack_f4_t5=STCK_F4_THETA5, stack_f5_p1=STCK_F5_PHI1,
                stack_3_site=STACK_3_SITE, stack_5_site=STACK_5_SITE,
                stack_bbvector_3=BBVECTOR_3, stack_bbvector_5=BBVECTOR_5,
                stack_f4_tB1=STCK_F4_THETAB1, stack_f4_tB2=STCK_F4_THETAB2)


def bonded_force(bond_type="backbone", temperature=296.15, average=True):
    force = OxDNABonded()
    params = dict(epsilon=FENE_EPS, r0=FENE_R0, delta=FENE_DELTA, pos_back=BACK_SITE,
                  pos_base=BASE_SITE, excl_eps=EXCL_EPS, bexc_base_base=EXCL[2],
                  bexc_base_back=EXCL[3], bexc_back_base=EXCL[4])
    params.update(stacking_params(temperature, average=average))
    force.params[bond_type] = params
    return force


def excluded_volume(nlist, types=DNA_BASES, r_cut=EXCVOL_R_CUT):
    force = ExcludedVolume(nlist=nlist, default_r_cut=r_cut, mode="none")
    pair = dict(eps=EXCL_EPS, base_site=BASE_SITE, back_site=BACK_SITE, back_back=EXCL[1],
                base_base=EXCL[2], base_back=EXCL[3], back_base=EXCL[4])
    for a, b in _all_pairs(types):
        force.params[(a, b)] = dict(pair)
    return force


def hb_epsilon(t1, t2, average=True):
    if average:
        return HYDR_EPS if dna1.is_complementary(t1, t2) else 0.0
    return HYDR_SEQ.get((t1, t2), 0.0)


def hydrogen_bonding(nlist, types=DNA_BASES, average=True, r_cut=HB_R_CUT):
    force = HydrogenBonding(nlist=nlist, default_r_cut=r_cut, mode="none")
    sf = (1.0 - math.exp(-(HYDR_RC - HYDR_R0) * HYDR_A)) ** 2
    f1 = (HYDR_A, HYDR_R0, HYDR_RLOW, HYDR_RHIGH, HYDR_RCLOW, HYDR_RCHIGH, HYDR_BLOW, HYDR_BHIGH)
    for a, b in _all_pairs(types):
        force.params[(a, b)] = dict(eps=hb_epsilon(a, b, average), shift_factor=sf,
                                    base_site=BASE_SITE, f1=f1, f4_t1=HB_F4_THETA1,
                                    f4_t23=HB_F4_THETA23, f4_t4=HB_F4_THETA4,
                                    f4_t78=HB_F4_THETA78)
    return force


def debye_params(t_kelvin=296.15, salt=DEFAULT_SALT):
    kT = dna1.kT_from_temperature(t_kelvin)
    lam = DH_LAMBDA_FACTOR * math.sqrt(kT / 0.1) / math.sqrt(salt)
    rhigh = 3.0 * lam
    q = DH_PREFACTOR
    b_smooth = -(math.exp(-rhigh / lam) * q * q * (rhigh + lam) ** 2) / (-4.0 * rhigh ** 3 * lam * lam * q)
    rc = rhigh * (q * rhigh + 3.0 * q * lam) / (q * (rhigh + lam))
    return -1.0 / lam, DH_PREFACTOR, b_smooth, rc, rhigh


def debye_huckel(nlist, types=DNA_BASES, t_kelvin=296.15, salt=DEFAULT_SALT, r_cut=None):
    mk, pref, b_smooth, rc, rhigh = debye_params(t_kelvin, salt)
    if r_cut is None:
        r_cut = rc + 2.0 * math.sqrt(sum(c * c for c in BACK_SITE))
    force = DebyeHuckel(nlist=nlist, default_r_cut=r_cut, mode="none")
    for a, b in _all_pairs(types):
        force.params[(a, b)] = dict(back_site=BACK_SITE, debye=(mk, pref, b_smooth, rc, rhigh))
    return force


def make_neighbor_list(buffer=0.4):
    return runtime.md.nlist.Cell(buffer=buffer, exclusions=("bond",))


def forces(nlist=None, temperature=296.15, salt=DEFAULT_SALT, average=True):
    """[bonded, excluded volume, hb, cross, coaxial, Debye] and the nlist."""
    if nlist is None:
        nlist = make_neighbor_list()
    return ([bonded_force(temperature=temperature, average=average), excluded_volume(nlist),
             hydrogen_bonding(nlist, average=average), cross_stacking(nlist),
             coaxial_stacking(nlist), debye_huckel(nlist, t_kelvin=temperature, salt=salt)],
            nlist)
