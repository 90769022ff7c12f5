// internal.h — helpers shared between the translation units of the library.
#pragma once

namespace pbf {

// Sets the message pbf_last_error(NULL) returns (thread-local).
void set_last_error(const char* msg);

}  // namespace pbf
