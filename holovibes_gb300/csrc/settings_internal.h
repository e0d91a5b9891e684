// Compute-settings documents as JSON values (settings.cpp), for the .holo footer (holo_file.cpp).
#pragma once

#include "hv_internal.h"
#include "json_lite.h"

namespace hv {

// Applies a compute-settings document over *s (lenient: keys unknown to this build are skipped).
hv_status settings_from_value(const json::Value& doc, hv_settings* s, bool lenient);
// The current-layout (v1) document of a settings record.
void settings_to_value(const hv_settings* s, json::Value& doc);
// Converts a compute-settings document to the current version in place; false if unknown.
bool settings_convert_to_current(json::Value& doc);
void settings_default(hv_settings* s);
hv_status settings_validate(hv_settings* s, const hv_frame_desc* fd);

}  // namespace hv
