// bignum_check.cpp -- test program for the pi program's host arithmetic
// (preclib_gb300/pi/bignum.cpp) on a schoolbook multiply backend, so the
// Newton division, square root and decimal conversion can be checked on a
// machine without a GPU.  Test infrastructure only: the pi program itself
// has no CPU multiply.
//
// One command per line on stdin, numbers in hexadecimal (no prefix, "0" for
// zero); one result line per command on stdout:
//   divmod N D          -> q r
//   divrecip N D extra  -> q r   (reciprocal of D at extra bits above the minimum)
//   isqrt N             -> s
//   dec N width         -> decimal digits
//   decpre N levels     -> decimal digits, powers built ahead for `levels` levels
#include <cstdio>
#include <iostream>
#include <sstream>
#include <string>

#include "../../preclib_gb300/pi/bignum.hpp"

using namespace precpi;

namespace {

struct SchoolBackend : MulBackend {
    void mul(const Nat& a, const Nat& b, Nat& out) override {
        out.d.assign(a.size() + b.size(), 0);
        if (!a.zero() && !b.zero()) mul_school(a.d.data(), a.size(), b.d.data(), b.size(), out.d.data());
        normalize(out);
    }
    void mul_many(const std::vector<const Nat*>& a, const std::vector<const Nat*>& b,
                  std::vector<Nat>& out) override {
        out.assign(a.size(), Nat());
        for (size_t i = 0; i < a.size(); ++i) mul(*a[i], *b[i], out[i]);
    }
};

Nat from_hex(const std::string& s) {
    Nat r;
    size_t bits = 0;
    for (size_t i = s.size(); i-- > 0;) {
        const char c = s[i];
        const u64 v = (u64)(c <= '9' ? c - '0' : (c | 32) - 'a' + 10);
        if (bits % 64 == 0) r.d.push_back(0);
        r.d.back() |= v << (bits % 64);
        bits += 4;
    }
    normalize(r);
    return r;
}

std::string to_hex(const Nat& x) {
    if (x.zero()) return "0";
    std::string s;
    char buf[17];
    std::snprintf(buf, sizeof buf, "%llx", (unsigned long long)x.d.back());
    s += buf;
    for (size_t i = x.size() - 1; i-- > 0;) {
        std::snprintf(buf, sizeof buf, "%016llx", (unsigned long long)x.d[i]);
        s += buf;
    }
    return s;
}

}  // namespace

int main() {
    SchoolBackend be;
    set_backend(&be);
    std::string line;
    while (std::getline(std::cin, line)) {
        std::istringstream in(line);
        std::string cmd, a, b;
        in >> cmd;
        if (cmd == "divmod" || cmd == "divrecip") {
            size_t extra = 0;
            in >> a >> b >> extra;
            const Nat N = from_hex(a), D = from_hex(b);
            Nat q, r;
            if (cmd == "divmod") {
                divmod(N, D, q, r);
            } else {
                const size_t nn = bitlen(N), nd = bitlen(D);
                const size_t P = (nn > nd ? nn - nd : 0) + 2 + 32 + extra;
                divmod_recip(N, D, recip(D, P), P, q, r);
            }
            std::cout << to_hex(q) << " " << to_hex(r) << "\n";
        } else if (cmd == "isqrt") {
            in >> a;
            std::cout << to_hex(isqrt(from_hex(a))) << "\n";
        } else if (cmd == "dec") {
            size_t width = 0;
            in >> a >> width;
            std::cout << to_decimal(from_hex(a), width) << "\n";
        } else if (cmd == "decpre") {
            int levels = 0;
            in >> a >> levels;
            const DecimalPowers pw = decimal_powers(levels);
            std::cout << to_decimal(from_hex(a), 0, &pw) << "\n";
        } else {
            std::cout << "?\n";
        }
        std::cout.flush();
    }
    return 0;
}
