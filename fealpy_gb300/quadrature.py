"""Symmetric quadrature rules on triangles and tetrahedra.

The rules are the ones FEALPy selects through ``TriangleMesh.quadrature_formula``
(``fealpy/mesh/triangle_mesh.py:80-98``, tables in ``fealpy/quadrature/triangle.py:15-329``)
and ``TetrahedronMesh.quadrature_formula`` (``fealpy/mesh/tetrahedron_mesh.py:144-163``,
tables in ``fealpy/quadrature/tetrahedron.py:6-243``).  They are published rules
(Williams, Shunn & Jameson 2014 for triangles; Keast-type rules for tetrahedra), and the
same points and weights are needed here because an under-integrated local matrix (for
example P2 mass with q=3) depends on the rule itself, not only on its degree.

Each rule is stored compactly as symmetry orbits ``(multiplicities, values, weight)``:
``values[k]`` is a barycentric coordinate that occurs ``multiplicities[k]`` times, and
the orbit expands to every distinct permutation of that coordinate tuple, each point
carrying ``weight``.  The decimal values are the published 15/16-digit constants.
"""
from itertools import permutations
from typing import Dict, List, Tuple

import numpy as np

__all__ = ["TriangleQuadrature", "TetrahedronQuadrature", "simplex_quadrature"]

_TRIANGLE_ORBITS = {
    1: [  # 1 points
        ((3,), (0.333333333333333,), 1.0),
    ],
    2: [  # 3 points
        ((2, 1), (0.166666666666667, 0.666666666666667), 0.333333333333333),
    ],
    3: [  # 6 points
        ((2, 1), (0.09157621350978, 0.81684757298044), 0.109951743655333),
        ((2, 1), (0.445948490915964, 0.108103018168071), 0.223381589678),
    ],
    4: [  # 10 points
        ((2, 1), (0.055564052669793, 0.888871894660413), 0.041955512996649),
        ((1, 1, 1), (0.634210747745723, 0.295533711735893, 0.070255540518384), 0.112098412070887),
        ((3,), (0.333333333333333,), 0.20154298858473),
    ],
    5: [  # 15 points
        ((2, 1), (0.035870877695734, 0.928258244608533), 0.017915455012303),
        ((2, 1), (0.241729395767967, 0.516541208464066), 0.127712195881265),
        ((2, 1), (0.474308787777079, 0.051382424445843), 0.076206062385535),
        ((1, 1, 1), (0.751183631106484, 0.2015038818818, 0.047312487011716), 0.055749810027115),
    ],
    6: [  # 21 points
        ((2, 1), (0.028112952182664, 0.943774095634672), 0.010359374696538),
        ((2, 1), (0.177139098469317, 0.645721803061365), 0.075394884326738),
        ((2, 1), (0.405508595867433, 0.188982808265134), 0.097547802373242),
        ((1, 1, 1), (0.817900980028499, 0.148565812270887, 0.033533207700614), 0.028969269372473),
        ((1, 1, 1), (0.604978911775132, 0.357196298615681, 0.037824789609186), 0.046046366595935),
    ],
    7: [  # 28 points
        ((2, 1), (0.019977187122193, 0.960045625755613), 0.005272170280495),
        ((2, 1), (0.131721767529998, 0.736556464940005), 0.044552936679504),
        ((3,), (0.333333333333333,), 0.083608212215637),
        ((2, 1), (0.485135346793461, 0.029729306413079), 0.033815712804198),
        ((1, 1, 1), (0.867911210117951, 0.107951981846011, 0.024136808036039), 0.015710461340183),
        ((1, 1, 1), (0.700872570380723, 0.270840772921567, 0.02828665669771), 0.028205136280616),
        ((1, 1, 1), (0.536654684206138, 0.316549598844617, 0.146795716949245), 0.06699595712783),
    ],
    8: [  # 36 points
        ((2, 1), (0.021171422779465, 0.95765715444107), 0.00563912378691),
        ((2, 1), (0.100584397395888, 0.798831205208225), 0.027148968192278),
        ((2, 1), (0.271038307711932, 0.457923384576135), 0.063100912533359),
        ((2, 1), (0.440191258403832, 0.119617483192335), 0.051752795679899),
        ((1, 1, 1), (0.879979641427232, 0.101763679498021, 0.018256679074748), 0.009866753574646),
        ((1, 1, 1), (0.582562022863673, 0.394033271669987, 0.023404705466341), 0.022008204800147),
        ((1, 1, 1), (0.751530614542782, 0.226245530909229, 0.022223854547989), 0.016644570076736),
        ((1, 1, 1), (0.635737183263105, 0.249079227621332, 0.115183589115563), 0.044326238118914),
    ],
    9: [  # 45 points
        ((2, 1), (0.078357605998763, 0.843284788002473), 0.017024468695001),
        ((2, 1), (0.220314093142718, 0.559371813714564), 0.045484616985315),
        ((2, 1), (0.4903209480069, 0.019358103986199), 0.016777583727179),
        ((1, 1, 1), (0.710726414278087, 0.19791878967951, 0.091354796042403), 0.029154505028877),
        ((1, 1, 1), (0.542373714730306, 0.360400011893839, 0.097226273375855), 0.037938703183624),
        ((2, 1), (0.017941506500789, 0.964116986998421), 0.004139739951845),
        ((1, 1, 1), (0.896950733986638, 0.089133098716849, 0.013916167296513), 0.006648325109921),
        ((1, 1, 1), (0.790422017699194, 0.191573237936673, 0.018004744364133), 0.010602381144458),
        ((1, 1, 1), (0.655463812371175, 0.326066002157021, 0.018470185471804), 0.014473600572032),
        ((2, 1), (0.386135747159797, 0.227728505680405), 0.052271893896168),
    ],
}

_TETRAHEDRON_ORBITS = {
    1: [  # 1 points
        ((4,), (0.25,), 1.0),
    ],
    2: [  # 4 points
        ((3, 1), (0.138196601125011, 0.585410196624968), 0.25),
    ],
    3: [  # 10 points
        ((3, 1), (0.0738349017262234, 0.77849529482133), 0.0476331348432089),
        ((2, 2), (0.406244343884051, 0.0937556561159491), 0.134911243437861),
    ],
    4: [  # 20 points
        ((3, 1), (0.0323525947272439, 0.902942215818268), 0.0070670747944695),
        ((2, 1, 1), (0.0603604415251421, 0.616596533061937, 0.262682583887779), 0.0469986689718877),
        ((3, 1), (0.309769304272862, 0.0706920871814129), 0.101936918289868),
    ],
    5: [  # 35 points
        ((3, 1), (0.0267367755543735, 0.91978967333688), 0.0021900463965388),
        ((2, 1, 1), (0.0391022406356488, 0.747759888481809, 0.174035630246894), 0.0143395670177665),
        ((2, 2), (0.454754599984483, 0.0452454000155172), 0.0250305395686746),
        ((2, 1, 1), (0.223201037962315, 0.503118645014598, 0.050479279060772), 0.0479839333057554),
        ((4,), (0.25,), 0.093174573119534),
    ],
    6: [  # 56 points
        ((3, 1), (0.0149520651530592, 0.955143804540822), 0.001037311233614),
        ((2, 1, 1), (0.0340960211962615, 0.77997600844154, 0.151831949165937), 0.009601664539948),
        ((2, 1, 1), (0.0462051504150017, 0.552655643106017, 0.354934056063979), 0.0164493976798232),
        ((2, 1, 1), (0.228190461068761, 0.538104322888002, 0.0055147549744775), 0.015374776651331),
        ((2, 1, 1), (0.352305260087994, 0.19618375957456, 0.099205720249453), 0.029352011837523),
        ((3, 1), (0.134478334792994, 0.596564995621017), 0.0366291366405108),
    ],
    7: [  # 84 points
        ((3, 1), (0.026878474414817, 0.919364576755549), 0.002144935144316),
        ((3, 1), (0.18714067580347, 0.438577972589591), 0.020826641690769),
        ((2, 2), (0.473575835127937, 0.026424164872063), 0.007210136064455),
        ((2, 2), (0.352045262027356, 0.147954737972644), 0.030798919159712),
        ((2, 1, 1), (0.020953442220056, 0.732309909692947, 0.22578320586694), 0.004357844813864),
        ((2, 1, 1), (0.096989733123466, 0.647557594086975, 0.158462939666092), 0.008593530677833),
        ((3, 1), (0.322111431830857, 0.033665704507429), 0.023000681669286),
        ((2, 1, 1), (0.097608162890442, 0.792939256469618, 0.011844417749498), 0.004863063904912),
        ((1, 1, 1, 1), (0.541184412800237, 0.296501020543124, 0.133558160703568, 0.028756405953071), 0.015595140078259),
    ],
}


def _expand(orbits) -> Tuple[np.ndarray, np.ndarray]:
    points: List[Tuple[float, ...]] = []
    weights: List[float] = []
    for mult, vals, w in orbits:
        base = []
        for m, v in zip(mult, vals):
            base.extend([v] * m)
        seen = set()
        for perm in permutations(base):
            if perm in seen:
                continue
            seen.add(perm)
            points.append(perm)
            weights.append(w)
    return np.asarray(points, dtype=np.float64), np.asarray(weights, dtype=np.float64)


_CACHE: Dict[Tuple[int, int], Tuple[np.ndarray, np.ndarray]] = {}


def simplex_quadrature(TD: int, q: int) -> Tuple[np.ndarray, np.ndarray]:
    """Barycentric points ``(NQ, TD+1)`` and weights ``(NQ,)`` of rule index ``q``.

    The weights sum to one (up to the rounding of the published decimals); the
    caller scales them by the signed cell measure, as FEALPy does.
    """
    key = (TD, q)
    if key not in _CACHE:
        table = {2: _TRIANGLE_ORBITS, 3: _TETRAHEDRON_ORBITS}.get(TD)
        if table is None:
            raise ValueError(f"no simplex quadrature for topological dimension {TD}")
        if q not in table:
            raise NotImplementedError(
                f"quadrature index {q} is not available for TD={TD} "
                f"(supported: {sorted(table)})")
        _CACHE[key] = _expand(table[q])
    bcs, ws = _CACHE[key]
    return bcs.copy(), ws.copy()


class _SimplexQuadrature:
    TD = 0

    def __init__(self, index: int, *, dtype=None, device=None):
        self.index = index
        self.quadpts, self.weights = simplex_quadrature(self.TD, index)

    def __len__(self):
        return self.weights.shape[0]

    def number_of_quadrature_points(self) -> int:
        return self.weights.shape[0]

    def get_quadrature_points_and_weights(self):
        return self.quadpts, self.weights

    def get_quadrature_point_and_weight(self, i: int):
        return self.quadpts[i], self.weights[i]


class TriangleQuadrature(_SimplexQuadrature):
    """Triangle rule by index, as ``fealpy.quadrature.TriangleQuadrature``."""
    TD = 2


class TetrahedronQuadrature(_SimplexQuadrature):
    """Tetrahedron rule by index, as ``fealpy.quadrature.TetrahedronQuadrature``."""
    TD = 3
