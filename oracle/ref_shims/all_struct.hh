// Stand-in for Backend/includes/struct/all_struct.hh in the comparison build: the JSON
// serialisation macros expand to nothing (no nlohmann_json), the enums and structs stay as declared.
#pragma once

#define SERIALIZE_JSON_STRUCT(Type, ...)
#define SERIALIZE_JSON_ENUM(Type, ...)
#define SETTING_RELATED_FUNCTIONS()
