// Minimal std::ostream insertion for GMP floats.
//
// Test infrastructure only (linked into oracle/_ref/sdpa_gmp by
// oracle/build_ref.sh).  The reference links -lgmpxx (Makefile.am:59),
// whose only out-of-line symbols it needs are the stream operators used by
// its rMessage/rError diagnostics (sdpa_tool.h:43-53).  The system provides
// libgmp.so.10 but no libgmpxx, so this file supplies the mpf/mpz/mpq
// inserters with gmp_printf-style formatting.  They only affect diagnostic
// text, never a computed value.
#include <gmp.h>
#include <ostream>
#include <string>

static std::string sdpg_fmt(const char *fmt, const void *x) {
    char *buf = nullptr;
    gmp_asprintf(&buf, fmt, x);
    std::string s(buf ? buf : "");
    void (*freefunc)(void *, size_t);
    mp_get_memory_functions(nullptr, nullptr, &freefunc);
    if (buf) freefunc(buf, s.size() + 1);
    return s;
}

std::ostream &operator<<(std::ostream &o, mpf_srcptr x) { return o << sdpg_fmt("%Fg", x); }
std::ostream &operator<<(std::ostream &o, mpz_srcptr x) { return o << sdpg_fmt("%Zd", x); }
std::ostream &operator<<(std::ostream &o, mpq_srcptr x) { return o << sdpg_fmt("%Qd", x); }
