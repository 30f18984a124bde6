"""The work partition of the whole-row fused step (launch form 6), checked on
the host without a GPU: the kernel's own schedule code (RowPieces, compiled
for the host as smat_row32_pieces) must give every cell of every plane to
exactly one CTA of an excitation, so that no two CTAs write one cell of the
new field set and none is left out (the fields are double-buffered, so reads
of the old set cannot race with writes).  Persistent groups (whole row tiles
in rounds, the leftover tiles' planes shared out) and z chunks, for grids and
group counts from one group to more groups than planes."""
import numpy as np
import pytest


def _cover(L1, L2, ty, zc, ngroups):
    from smatranem_gb300 import fdtd as f
    nyt = -(-L1 // ty)
    zcc = min(zc, L2)
    items = nyt * -(-L2 // zcc) if zcc > 0 else max(ngroups, 1)
    cover = np.zeros((L1, L2), np.int32)
    npieces = []
    for g in range(items):
        pieces = f.row32_pieces(L1, L2, ty, zc, ngroups, g)
        npieces.append(len(pieces))
        for yt, z0, z1 in pieces:
            assert 0 <= yt < nyt and 0 <= z0 < z1 <= L2, (yt, z0, z1)
            y0 = yt * ty
            cover[y0:min(y0 + ty, L1), z0:z1] += 1
    return cover, npieces


@pytest.mark.parametrize("L1,L2", [(192, 160), (17, 19), (1, 1), (5, 3), (640, 512), (13, 47), (24, 1)])
@pytest.mark.parametrize("ty", [1, 2, 5, 7, 16])
def test_persistent_groups_partition_the_grid(built, L1, L2, ty):
    for ngroups in sorted({0, 1, 2, 3, 7, 19, 38, 152, 1000}):
        cover, npieces = _cover(L1, L2, ty, 0, ngroups)
        assert np.all(cover == 1), (L1, L2, ty, ngroups, np.argwhere(cover != 1)[:4])
        # whole tiles in rounds, then at most a few pieces of the leftover tiles' planes
        nyt = -(-L1 // ty)
        G = max(ngroups, 1)
        assert max(npieces) <= nyt // G + 2 + (nyt % G > 0)


@pytest.mark.parametrize("L1,L2", [(192, 160), (17, 19), (1, 1), (5, 3), (13, 47)])
@pytest.mark.parametrize("ty,zc", [(1, 1), (2, 5), (5, 20), (4, 40), (3, 1000), (16, 7)])
def test_z_chunks_partition_the_grid(built, L1, L2, ty, zc):
    cover, npieces = _cover(L1, L2, ty, zc, 0)
    assert np.all(cover == 1)
    assert set(npieces) == {1}


def test_bad_arguments_are_refused(built):
    from smatranem_gb300 import fdtd as f
    for args in [(0, 5, 2, 0, 4, 0), (5, 0, 2, 0, 4, 0), (5, 5, 0, 0, 4, 0), (5, 5, 2, -1, 4, 0),
                 (5, 5, 2, 0, 4, 4), (5, 5, 2, 0, -1, 0), (5, 5, 2, 2, 0, 9)]:
        with pytest.raises(f.FdtdError):
            f.row32_pieces(*args)
