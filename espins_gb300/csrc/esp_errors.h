// Error message of calls that have no handle (esp_api.cu).
#pragma once

namespace esp {
// printf-style; writes into a fixed buffer read by esp_last_error(NULL, ...).
void set_global_error(const char *fmt, ...);
}  // namespace esp
