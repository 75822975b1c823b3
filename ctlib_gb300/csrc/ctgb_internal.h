// Internal declarations shared by the translation units of libctgb.so.
#ifndef CTGB_INTERNAL_H
#define CTGB_INTERNAL_H

#include <string>

namespace ctgb {
// records `msg` as the calling thread's last error (ctgb_last_error) and
// returns `code`
int fail(int code, const std::string& msg);
}  // namespace ctgb

#endif
