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

// HPP: a head-on pair swaps to the perpendicular pair when the other pair is
// empty.  The chirality is not used.
LGCA_HDI void collide_hpp(uint64_t n[4])
{
    const uint64_t h02 = n[0] & n[2] & ~(n[1] | n[3]);
    const uint64_t h13 = n[1] & n[3] & ~(n[0] | n[2]);
    const uint64_t ch = h02 | h13;
    n[0] ^= ch; n[1] ^= ch; n[2] ^= ch; n[3] ^= ch;
}

// FHP-I (REST = false) and FHP-II/III (REST = true).  `p` is the chirality
// word: 1 rotates a two-body collision one way, 0 the other.
template <bool REST>
LGCA_HDI void collide_fhp(uint64_t n[7], uint64_t p)
{
    const uint64_t a = n[1], b = n[2], c = n[3], d = n[4], e = n[5], f = n[0];
    const uint64_t np = ~p;

    // head-on pairs with all other moving channels empty
    const uint64_t db1 = a & d & ~(b | c | e | f);
    const uint64_t db2 = b & e & ~(a | c | d | f);
    const uint64_t db3 = c & f & ~(a | b | d | e);
    // symmetric three-body a,c,e <-> b,d,f (alternating occupation)
    const uint64_t triple = (a ^ b) & (b ^ c) & (c ^ d) & (d ^ e) & (e ^ f);

    uint64_t cha = triple | db1 | (p & db2) | (np & db3);
    uint64_t chb = triple | db2 | (p & db3) | (np & db1);
    uint64_t chc = triple | db3 | (p & db1) | (np & db2);
    uint64_t chd = cha, che = chb, chf = chc;

    if (REST) {
        const uint64_t r = n[6];
        // exactly one moving particle x: x & ~(the other five)
        const uint64_t bcdef = b | c | d | e | f;
        const uint64_t oa = a & ~bcdef;
        const uint64_t ob = b & ~(a | c | d | e | f);
        const uint64_t oc = c & ~(a | b | d | e | f);
        const uint64_t od = d & ~(a | b | c | e | f);
        const uint64_t oe = e & ~(a | b | c | d | f);
        const uint64_t of = f & ~(a | b | c | d | e);
        // rest + one moving -> two moving at +-60 degrees
        const uint64_t ra = r & oa, rb = r & ob, rc = r & oc;
        const uint64_t rd = r & od, re = r & oe, rf = r & of;
        // two moving at 120 degrees apart, no rest -> rest + one moving
        const uint64_t nr = ~r;
        const uint64_t ra2 = f & b & nr & ~(a | c | d | e);
        const uint64_t rb2 = a & c & nr & ~(b | d | e | f);
        const uint64_t rc2 = b & d & nr & ~(a | c | e | f);
        const uint64_t rd2 = c & e & nr & ~(a | b | d | f);
        const uint64_t re2 = d & f & nr & ~(a | b | c | e);
        const uint64_t rf2 = e & a & nr & ~(b | c | d | f);

        cha |= ra | rb | rf | ra2 | rb2 | rf2;
        chd |= rd | rc | re | rd2 | rc2 | re2;
        chb |= rb | ra | rc | rb2 | ra2 | rc2;
        che |= re | rd | rf | re2 | rd2 | rf2;
        chc |= rc | rb | rd | rc2 | rb2 | rd2;
        chf |= rf | ra | re | rf2 | ra2 | re2;
        const uint64_t chr = ra | rb | rc | rd | re | rf | ra2 | rb2 | rc2 | rd2 | re2 | rf2;
        n[6] = r ^ chr;
    }
    n[1] = a ^ cha; n[2] = b ^ chb; n[3] = c ^ chc;
    n[4] = d ^ chd; n[5] = e ^ che; n[0] = f ^ chf;
}

template <int MODEL>
LGCA_HDI void collide(uint64_t *n, uint64_t p)
{
    if (MODEL == M_HPP) collide_hpp(n);
    else if (MODEL == M_FHP_I) collide_fhp<false>(n, p);
    else collide_fhp<true>(n, p);
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
