// block_lists.h — the (128-row block, 32-wide k block) pairs of B that touch a stored tile.
//
// B is stored as the 64 x 64 tiles (I >= J) that hold a Schwarz-significant pair; the
// tensor-core forms copy B into 128 x 32 operand blocks of the dense square, and keep (and
// multiply) only the blocks that intersect a stored tile or its mirror.  Lists are grouped
// by 128-row block: block kb of row block mb is listed at kbs[ptr[mb] .. ptr[mb+1]).
#pragma once

#include <vector>

namespace gdfjk {

struct BlockLists {
    std::vector<int> ptr;  // nmb + 1
    std::vector<int> kb;   // listed k block of each entry
    std::vector<int> mb;   // row block of each entry
};

// map_host: [nT * nT] stored-tile index of (I, J), I >= J, -1 if absent
inline BlockLists build_block_lists(const int* map_host, int nT, int nbf_p, int rows_per_block, int k_per_block,
                                    int tile) {
    BlockLists bl;
    const int nmb = nbf_p / rows_per_block, nkb = nbf_p / k_per_block;
    const int tiles_per_mb = rows_per_block / tile;
    bl.ptr.assign(nmb + 1, 0);
    for (int mb = 0; mb < nmb; ++mb) {
        for (int kb = 0; kb < nkb; ++kb) {
            const int J = (kb * k_per_block) / tile;
            bool any = false;
            for (int I = tiles_per_mb * mb; I < tiles_per_mb * (mb + 1) && !any; ++I)
                if (I < nT && J < nT) any = map_host[(I >= J ? I : J) * nT + (I >= J ? J : I)] >= 0;
            if (any) {
                bl.kb.push_back(kb);
                bl.mb.push_back(mb);
            }
        }
        bl.ptr[mb + 1] = (int)bl.kb.size();
    }
    return bl;
}

}  // namespace gdfjk
