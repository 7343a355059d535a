"""oxDNA2 model: grooved BACK site, updated constants and Debye-Hueckel.

Same public names, constants and signatures as the reference's
``oxdna/model/dna2.py``; cross-stacking and the f1..f5 shapes are shared with
:mod:`oxdna.model.dna1`.
"""

import itertools
import math

from .. import runtime
from ..forces import (CoaxialStacking, DebyeHuckel, ExcludedVolume, HBondCross,
                      HydrogenBonding, OxDNABonded)
from ..io import DNA_BASES
from . import dna1

POS_MM_BACK1, POS_MM_BACK2 = -0.3400, 0.3408
BACK_SITE = (POS_MM_BACK1, POS_MM_BACK2, 0.0)

FENE_R0 = 0.7564
STCK_BASE_EPS = 1.3523
STCK_FACT_EPS = 2.6717
HYDR_EPS = 1.0678

STCK_FACT_EPS_SEQ = 0.18
STCK_SEQ = {
    ("G", "C"): 1.69339, ("C", "G"): 1.74669, ("G", "G"): 1.61295, ("C", "C"): 1.61295,
    ("G", "A"): 1.59887, ("T", "C"): 1.59887, ("A", "G"): 1.61898, ("C", "T"): 1.61898,
    ("T", "G"): 1.66322, ("C", "A"): 1.66322, ("G", "T"): 1.68032, ("A", "C"): 1.68032,
    ("A", "T"): 1.56166, ("T", "A"): 1.64311, ("A", "A"): 1.84642, ("T", "T"): 1.58952,
}
HYDR_SEQ = {("A", "T"): 0.88537, ("T", "A"): 0.88537, ("C", "G"): 1.23238, ("G", "C"): 1.23238}

CXST_K = 58.5
CXST_F4_THETA1 = (2.0, 10.9032, math.pi - 0.25, 0.65, 0.769231)
CXST_THETA1_SA = 20.0
CXST_THETA1_SB = math.pi - 0.1 * (math.pi - (math.pi - 0.25))

DH_LAMBDA_FACTOR = 0.3616455
DH_PREFACTOR = 0.0543
DEFAULT_SALT = 0.5


def stacking_eps_table(t_kelvin=296.15):
    eps = STCK_BASE_EPS + STCK_FACT_EPS * dna1.kT_from_temperature(t_kelvin)
    return [[eps] * 4 for _ in range(4)]


def sequence_stacking_eps_table(t_kelvin=296.15):
    kT = dna1.kT_from_temperature(t_kelvin)
    factor = 1.0 - STCK_FACT_EPS_SEQ + kT * 9.0 * STCK_FACT_EPS_SEQ
    return [[STCK_SEQ[(a, b)] * factor for b in DNA_BASES] for a in DNA_BASES]


def _stacking_params(t_kelvin, average=True):
    sp = dna1.stacking_params(t_kelvin)
    table = stacking_eps_table(t_kelvin) if average else sequence_stacking_eps_table(t_kelvin)
    sp["stack_eps"] = tuple(table[i][j] for i in range(4) for j in range(4))
    return sp


def bonded_force(bond_type="backbone", temperature=296.15, stacking=True, average=True):
    force = OxDNABonded()
    params = dict(epsilon=dna1.FENE_EPS, r0=FENE_R0, delta=dna1.FENE_DELTA, pos_back=BACK_SITE,
                  pos_base=dna1.BASE_SITE, excl_eps=dna1.EXCL_EPS,
                  bexc_base_base=dna1.EXCL[2], bexc_base_back=dna1.EXCL[3],
                  bexc_back_base=dna1.EXCL[4])
    if stacking:
        params.update(_stacking_params(temperature, average=average))
    force.params[bond_type] = params
    return force


def _all_pairs(types):
    return itertools.combinations_with_replacement(types, 2)


def excluded_volume(nlist, types=DNA_BASES, r_cut=dna1.EXCVOL_R_CUT):
    force = ExcludedVolume(nlist=nlist, default_r_cut=r_cut, mode="none")
    pair = dict(eps=dna1.EXCL_EPS, base_site=dna1.BASE_SITE, back_site=BACK_SITE,
                back_back=dna1.EXCL[1], base_base=dna1.EXCL[2], base_back=dna1.EXCL[3],
                back_base=dna1.EXCL[4])
    for a, b in _all_pairs(types):
        force.params[(a, b)] = dict(pair)
    return force


def hb_epsilon(t1, t2, average=True):
    if average:
        return HYDR_EPS if dna1.is_complementary(t1, t2) else 0.0
    return HYDR_SEQ.get((t1, t2), 0.0)


def hydrogen_bonding(nlist, types=DNA_BASES, average=True, r_cut=dna1.HB_R_CUT):
    force = HydrogenBonding(nlist=nlist, default_r_cut=r_cut, mode="none")
    for a, b in _all_pairs(types):
        force.params[(a, b)] = dict(
            eps=hb_epsilon(a, b, average), shift_factor=dna1.hb_shift_factor(),
            base_site=dna1.BASE_SITE, f1=dna1._hb_f1(), f4_t1=dna1.HB_F4_THETA1,
            f4_t23=dna1.HB_F4_THETA23, f4_t4=dna1.HB_F4_THETA4, f4_t78=dna1.HB_F4_THETA78)
    return force


def hbond_cross(nlist, types=DNA_BASES, average=True, r_cut=None):
    if r_cut is None:
        r_cut = max(dna1.HB_R_CUT, dna1.CROSS_R_CUT)
    force = HBondCross(nlist=nlist, default_r_cut=r_cut, mode="none")
    for a, b in _all_pairs(types):
        force.params[(a, b)] = dict(
            base_site=dna1.BASE_SITE, eps=hb_epsilon(a, b, average),
            shift_factor=dna1.hb_shift_factor(), f1=dna1._hb_f1(),
            hb_f4_t1=dna1.HB_F4_THETA1, hb_f4_t23=dna1.HB_F4_THETA23,
            hb_f4_t4=dna1.HB_F4_THETA4, hb_f4_t78=dna1.HB_F4_THETA78, f2=dna1.CRST_F2,
            cs_f4_t1=dna1.CRST_F4_THETA1, cs_f4_t23=dna1.CRST_F4_THETA23,
            cs_f4_t4=dna1.CRST_F4_THETA4, cs_f4_t78=dna1.CRST_F4_THETA78)
    return force


def coaxial_stacking(nlist, types=DNA_BASES, r_cut=dna1.COAX_R_CUT):
    force = CoaxialStacking(nlist=nlist, default_r_cut=r_cut, mode="none")
    pair = dict(stack_site=dna1.STACK_SITE, stack_back_ref=dna1.STACK_BACK_REF, gamma=dna1.GAMMA,
                f2=(CXST_K,) + dna1.CXST_F2[1:], f4_t1=CXST_F4_THETA1, f4_t4=dna1.CXST_F4_THETA4,
                f4_t56=dna1.CXST_F4_THETA56, f5_phi3=dna1.CXST_F5_PHI3, t1_mode=1,
                t1_sa=CXST_THETA1_SA, t1_sb=CXST_THETA1_SB, phi3_enabled=False)
    for a, b in _all_pairs(types):
        force.params[(a, b)] = dict(pair)
    return force


def debye_params(t_kelvin=296.15, salt=DEFAULT_SALT):
    """(minus_kappa, prefactor, b_smooth, rc, rhigh) of the Debye-Hueckel term."""
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
        r_cut = rc + 2.0 * math.sqrt(POS_MM_BACK1 ** 2 + POS_MM_BACK2 ** 2)
    force = DebyeHuckel(nlist=nlist, default_r_cut=r_cut, mode="none")
    for a, b in _all_pairs(types):
        force.params[(a, b)] = dict(back_site=BACK_SITE, debye=(mk, pref, b_smooth, rc, rhigh))
    return force


def make_neighbor_list(buffer=0.4):
    return runtime.md.nlist.Cell(buffer=buffer, exclusions=("bond",))


def forces(nlist=None, temperature=296.15, salt=DEFAULT_SALT, fused=False, average=True):
    """[bonded, excluded volume, (hb, cross) or hbcross, coaxial, Debye] and the nlist."""
    if nlist is None:
        nlist = make_neighbor_list()
    base_base = ([hbond_cross(nlist, average=average)] if fused
                 else [hydrogen_bonding(nlist, average=average), dna1.cross_stacking(nlist)])
    return ([bonded_force(temperature=temperature, average=average), excluded_volume(nlist),
             *base_base, coaxial_stacking(nlist),
             debye_huckel(nlist, t_kelvin=temperature, salt=salt)], nlist)
