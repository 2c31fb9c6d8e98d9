// Bit-sliced lattice-gas collision rules.
//
// Each argument is one 64-bit word of a channel bit-plane: bit i of `n[d]`
// is the occupation of channel d at site x0 + i.  The rules are the
// reference's per-cell boolean rules (keva92/lgca src/lgca_models.h) applied
// to 64 sites at once: a per-cell `&`, `|`, `^` on 0/1 values is the same
// operation on every bit of a word, and the reference's `~p` on the 0/1
// chirality is the complement of the chirality word.
//
//   HPP      src/lgca_models.h:134-152  head-on pairs (0,2) <-> (1,3)
//   FHP-I    src/lgca_models.h:367-395  two-body head-on (rotated by the
//            chirality) and symmetric three-body
//   FHP-II   src/lgca_models.h:568-613  FHP-I + rest-particle rules
//   FHP-III  src/lgca_models.h:786-856  identical to FHP-II: every extra
//            term ANDs a two-body pattern that requires a channel to be empty
//            with a term that requires it occupied, so all of them are zero.
//            The two models share one function (checked exhaustively against
//            the reference in the tests).
//
// Channel letters follow the reference: a..f = channels 1,2,3,4,5,0 and
// r = rest channel 6.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define LGCA_HDI __host__ __device__ __forceinline__
#define LGCA_HDM __host__ __device__
#else
#define LGCA_HDI static inline
#define LGCA_HDM
#endif

namespace lgca_gpu {

enum : int { M_HPP = 0, M_FHP_I = 1, M_FHP_II = 2, M_FHP_III = 3 };

template <int MODEL> struct ModelTraits;
template <> struct ModelTraits<M_HPP> { static constexpr int D = 4; };
template <> struct ModelTraits<M_FHP_I> { static constexpr int D = 6; };
template <> struct ModelTraits<M_FHP_II> { static constexpr int D = 7; };
template <> struct ModelTraits<M_FHP_III> { static constexpr int D = 7; };

// The rules below work on words of any unsigned type Word (64 or 32 sites).
//
// HPP: a head-on pair swaps to the perpendicular pair when the other pair is
// empty.  The chirality is not used.  The state is exactly {0, 2} or exactly
// {1, 3} when n0 != n1, n0 == n2 and n1 == n3.
template <class Word = uint64_t>
LGCA_HDI void collide_hpp(Word n[4])
{
    const Word ch = (n[0] ^ n[1]) & ~(n[0] ^ n[2]) & ~(n[1] ^ n[3]);
    n[0] ^= ch; n[1] ^= ch; n[2] ^= ch; n[3] ^= ch;
}

// FHP-I (REST = false) and FHP-II/III (REST = true).  `p` is the chirality
// word: 1 rotates a two-body collision one way, 0 the other.
//
// The reference writes every collision pattern as "these channels occupied
// and all other moving channels empty" (e.g. db1 = a&d&~(b|c|e|f),
// src/lgca_models.h:376) and flips channel x when any pattern that moves x
// matches.  The same boolean function, regrouped for few operations, indexing
// the moving channels n0..n5 around the hexagon (the reference's a..f are
// n1..n5, n0):
//   * count the occupied moving channels of each half-hexagon with a full
//     adder (s = parity, k = carry: the half's count is s + 2k) and form
//     "exactly 1 / 2 / 3 moving" masks straight from the two halves:
//       1: s1 != s2 and no carry;  3: s1 != s2 and exactly one carry;
//       2: s1 == s2 == 1 and no carry, or s1 == s2 == 0 and exactly one carry;
//   * head-on pair k = {n_k, n_k+3}: P_k = n_k & n_k+3 & is2; the pair turns by
//     -60 deg (p = 1) or +60 deg (p = 0), so channel pair k flips when P_k or
//     (p ? P_k+1 : P_k-1) holds (the reference's db1|(p&db2)|(~p&db3));
//   * three-body: with exactly three moving, (n0 n2 n4) or (n1 n3 n5) is full
//     exactly when n0 == n2 == n4; then T flips all six;
//   * rest rules (FHP-II): a rest particle plus a single moving particle at x
//     (R1 = r & is1) and two moving particles at x-1, x+1 without rest
//     (R2 = ~r & is2) both have their "centre" at x:
//       K_x = (R1 & n_x) | (R2 & n_x-1 & n_x+1),
//     and flip exactly channels x-1, x, x+1 and the rest channel.
// Checked exhaustively against the reference rules in the tests.
template <bool REST, class Word = uint64_t>
LGCA_HDI void collide_fhp(Word n[7], Word p)
{
    const Word n0 = n[0], n1 = n[1], n2 = n[2], n3 = n[3], n4 = n[4], n5 = n[5];

    // half-hexagon counts: s + 2k for (n0, n1, n2) and (n3, n4, n5)
    const Word s1 = n0 ^ n1 ^ n2, k1 = (n0 & n1) | (n2 & (n0 ^ n1));
    const Word s2 = n3 ^ n4 ^ n5, k2 = (n3 & n4) | (n5 & (n3 ^ n4));
    const Word sx = s1 ^ s2;
    const Word is3 = sx & (k1 ^ k2);
    const Word is2 = ~sx & ((s1 & ~(k1 | k2)) | (~s1 & (k1 ^ k2)));

    const Word P0 = n0 & n3 & is2, P1 = n1 & n4 & is2, P2 = n2 & n5 & is2;
    const Word T = is3 & ~((n0 ^ n2) | (n2 ^ n4));
    const Word X0 = T | P0 | ((p & P1) | (~p & P2));
    const Word X1 = T | P1 | ((p & P2) | (~p & P0));
    const Word X2 = T | P2 | ((p & P0) | (~p & P1));

    if (REST) {
        const Word r = n[6];
        const Word is1 = sx & ~(k1 | k2);
        const Word R1 = r & is1, R2 = ~r & is2;
        const Word K0 = (R1 & n0) | (R2 & n5 & n1);
        const Word K1 = (R1 & n1) | (R2 & n0 & n2);
        const Word K2 = (R1 & n2) | (R2 & n1 & n3);
        const Word K3 = (R1 & n3) | (R2 & n2 & n4);
        const Word K4 = (R1 & n4) | (R2 & n3 & n5);
        const Word K5 = (R1 & n5) | (R2 & n4 & n0);
        n[0] = n0 ^ (X0 | K5 | K0 | K1);
        n[1] = n1 ^ (X1 | K0 | K1 | K2);
        n[2] = n2 ^ (X2 | K1 | K2 | K3);
        n[3] = n3 ^ (X0 | K2 | K3 | K4);
        n[4] = n4 ^ (X1 | K3 | K4 | K5);
        n[5] = n5 ^ (X2 | K4 | K5 | K0);
        n[6] = r ^ ((K0 | K1 | K2) | (K3 | K4 | K5));
    } else {
        n[0] = n0 ^ X0; n[3] = n3 ^ X0;
        n[1] = n1 ^ X1; n[4] = n4 ^ X1;
        n[2] = n2 ^ X2; n[5] = n5 ^ X2;
    }
}

template <int MODEL, class Word>
LGCA_HDI void collide_w(Word *n, Word p)
{
    if (MODEL == M_HPP) collide_hpp<Word>(n);
    else if (MODEL == M_FHP_I) collide_fhp<false, Word>(n, p);
    else collide_fhp<true, Word>(n, p);
}
template <int MODEL>
LGCA_HDI void collide(uint64_t *n, uint64_t p)
{
    collide_w<MODEL, uint64_t>(n, p);
}

// Inverse and mirror direction tables (src/lgca_models.h:44-48 HPP,
// :239-243 FHP-I, :446-450 and :664-668 FHP-II/III) as index functions:
//   HPP  INV {2,3,0,1}   MIR_X {0,3,2,1}   MIR_Y {2,1,0,3}
//   FHP  INV {3,4,5,0,1,2,6}   MIR_X {0,5,4,3,2,1,6}   MIR_Y {3,2,1,0,5,4,6}
template <int MODEL> struct Dirs {
    LGCA_HDM static constexpr int inv(int d)
    {
        return MODEL == M_HPP ? ((d + 2) & 3) : (d == 6 ? 6 : (d + 3) % 6);
    }
    LGCA_HDM static constexpr int mirx(int d)
    {
        return MODEL == M_HPP ? ((4 - d) & 3) : (d == 6 ? 6 : (6 - d) % 6);
    }
    LGCA_HDM static constexpr int miry(int d)
    {
        return MODEL == M_HPP ? ((6 - d) & 3) : (d == 6 ? 6 : (d < 4 ? 3 - d : 9 - d));
    }
};

}  // namespace lgca_gpu
