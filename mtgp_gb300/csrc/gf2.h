// gf2.h -- host-side GF(2)[x] arithmetic for jump polynomials.
//
// Replaces the NTL calls the reference uses offline: MinPolySeq for the
// characteristic polynomial (mtgp32-calc-poly.cpp:36-45) and PowerXMod for
// jump polynomials (mtgp-calc-jump.hpp:135-162).  Polynomials are vectors of
// 64-bit words, bit i of the vector = coefficient of X^i.  Portable C++ (no
// carry-less-multiply intrinsics), identical results on every host.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace mtgp {
namespace gf2 {

using Poly = std::vector<uint64_t>;

int degree(const Poly &p);                       // -1 for the zero polynomial
Poly mul(const Poly &a, const Poly &b);          // a * b
void reduce(Poly &p, const Poly &m, int dm);     // p mod m, in place
Poly mulmod(const Poly &a, const Poly &b, const Poly &m, int dm);
Poly sqrmod(const Poly &a, const Poly &m, int dm);
// X^e mod m; e is little-endian 32-bit words (through Modulus).
Poly powxmod(const std::vector<uint32_t> &e, const Poly &m, int dm);
// Arithmetic modulo one fixed polynomial m of degree dm, with precomputed
// tables (about 2.9 MB for dm = 11213): reduction clears eight coefficients
// per table XOR, and products use the 8-bit comb method.
class Modulus {
  public:
    Modulus(const Poly &m, int dm);
    int degree() const { return dm_; }
    int words() const { return (dm_ + 63) / 64; }  // words of a reduced polynomial
    void reduce(Poly &p) const;                     // p mod m, in place
    Poly mulmod(const Poly &a, const Poly &b) const;
    Poly sqrmod(const Poly &a) const;
    Poly powx(const std::vector<uint32_t> &e) const;  // X^e mod m

  private:
    Poly m_;
    int dm_, tw_;
    // tab_[(a * 256 + b) * tw_ ..]: (q_b * m) << 8a, where q_b (degree < 8) is
    // the quotient that clears the eight coefficients dm .. dm+7 equal to b
    std::vector<uint64_t> tab_;
};
Poly mulComb(const Poly &a, const Poly &b);  // a * b, 8-bit comb
// floor(X^e / m) for m of degree dm <= e (long division), e.g. the Barrett
// constant floor(X^(2 dm) / m).
Poly divXpow(int e, const Poly &m, int dm);

// Minimal polynomial of the bit sequence s (Berlekamp-Massey); returns the
// degree L and writes chi (monic, degree L).
int minpoly(const std::vector<uint8_t> &s, Poly *chi);
// uint32-array form of the reference (mtgp-calc-jump.hpp:67-91).
std::vector<uint32_t> toWords32(const Poly &p, int nwords);
Poly fromWords32(const uint32_t *w, int nwords);
// Hex form of the reference (mtgp-calc-jump.hpp:34-58, 98-126).
bool fromHex(const char *s, Poly *p, int *ncoef);
std::string toHex(const Poly &p);

}  // namespace gf2
}  // namespace mtgp
