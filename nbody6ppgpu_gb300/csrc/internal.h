// Functions shared between the library's translation units (not exported).
#pragma once

namespace gpunb {
// record an error in the gpunb_last_error() slot and apply the abort policy
void report_failure(int code, const char *msg);
}  // namespace gpunb
