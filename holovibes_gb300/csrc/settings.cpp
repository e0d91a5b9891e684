// Compute-settings JSON: a small JSON reader, the reference's ComputeSettings key layout with its
// default values, partial-merge loading and the TransformApi validation rules.
//
// Reference behaviour (Holovibes):
//   load / merge   Backend/sources/core/compute_settings.cc:24-99 (merge_json: every key of the
//                  document must exist in the default ComputeSettings, objects merge recursively)
//   layout         Backend/includes/struct/{compute_settings,rendering,view,composite,advanced}_struct.hh
//   defaults       Backend/includes/core/holovibes.hh:370-450
//   enum strings   Backend/includes/enum/enum_space_transformation.hh:32-41, enum_time_transformation.hh:24-30,
//                  enum_img_type.hh:28-37
//   validation     Backend/sources/api/transform_api.cc:16-206
#include <cctype>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "hv_internal.h"

namespace hv {
namespace json {

struct Value
{
    enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
    bool b = false;
    double num = 0.0;
    std::string str;
    std::vector<Value> arr;
    std::vector<std::pair<std::string, Value>> obj;  // insertion order

    const Value* find(const std::string& k) const
    {
        for (const auto& kv : obj)
            if (kv.first == k)
                return &kv.second;
        return nullptr;
    }
    Value* find(const std::string& k)
    {
        for (auto& kv : obj)
            if (kv.first == k)
                return &kv.second;
        return nullptr;
    }
};

struct Parser
{
    const char* p;
    const char* end;
    std::string err;

    void ws()
    {
        while (p < end && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r'))
            ++p;
    }
    bool fail(const char* m)
    {
        if (err.empty())
            err = m;
        return false;
    }
    bool lit(const char* s)
    {
        const size_t n = std::strlen(s);
        if (static_cast<size_t>(end - p) < n || std::strncmp(p, s, n) != 0)
            return false;
        p += n;
        return true;
    }
    bool string(std::string& out)
    {
        if (p >= end || *p != '"')
            return fail("expected string");
        ++p;
        while (p < end && *p != '"')
        {
            char c = *p++;
            if (c == '\\')
            {
                if (p >= end)
                    return fail("bad escape");
                const char e = *p++;
                switch (e)
                {
                case '"': out += '"'; break;
                case '\\': out += '\\'; break;
                case '/': out += '/'; break;
                case 'b': out += '\b'; break;
                case 'f': out += '\f'; break;
                case 'n': out += '\n'; break;
                case 'r': out += '\r'; break;
                case 't': out += '\t'; break;
                case 'u':
                {
                    if (end - p < 4)
                        return fail("bad unicode escape");
                    unsigned int cp = 0;
                    for (int i = 0; i < 4; ++i)
                    {
                        const char h = p[i];
                        cp <<= 4;
                        if (h >= '0' && h <= '9')
                            cp |= static_cast<unsigned int>(h - '0');
                        else if (h >= 'a' && h <= 'f')
                            cp |= static_cast<unsigned int>(h - 'a' + 10);
                        else if (h >= 'A' && h <= 'F')
                            cp |= static_cast<unsigned int>(h - 'A' + 10);
                        else
                            return fail("bad unicode escape");
                    }
                    p += 4;
                    if (cp < 0x80)
                        out += static_cast<char>(cp);
                    else if (cp < 0x800)
                    {
                        out += static_cast<char>(0xC0 | (cp >> 6));
                        out += static_cast<char>(0x80 | (cp & 0x3F));
                    }
                    else
                    {
                        out += static_cast<char>(0xE0 | (cp >> 12));
                        out += static_cast<char>(0x80 | ((cp >> 6) & 0x3F));
                        out += static_cast<char>(0x80 | (cp & 0x3F));
                    }
                    break;
                }
                default: return fail("bad escape");
                }
            }
            else
                out += c;
        }
        if (p >= end)
            return fail("unterminated string");
        ++p;
        return true;
    }
    bool value(Value& v, int depth)
    {
        if (depth > 64)
            return fail("nesting too deep");
        ws();
        if (p >= end)
            return fail("unexpected end");
        const char c = *p;
        if (c == '{')
        {
            ++p;
            v.kind = Value::Object;
            ws();
            if (p < end && *p == '}')
            {
                ++p;
                return true;
            }
            for (;;)
            {
                ws();
                std::string k;
                if (!string(k))
                    return false;
                ws();
                if (p >= end || *p != ':')
                    return fail("expected ':'");
                ++p;
                Value child;
                if (!value(child, depth + 1))
                    return false;
                Value* existing = v.find(k);
                if (existing)
                    *existing = std::move(child);
                else
                    v.obj.emplace_back(std::move(k), std::move(child));
                ws();
                if (p < end && *p == ',')
                {
                    ++p;
                    continue;
                }
                if (p < end && *p == '}')
                {
                    ++p;
                    return true;
                }
                return fail("expected ',' or '}'");
            }
        }
        if (c == '[')
        {
            ++p;
            v.kind = Value::Array;
            ws();
            if (p < end && *p == ']')
            {
                ++p;
                return true;
            }
            for (;;)
            {
                Value child;
                if (!value(child, depth + 1))
                    return false;
                v.arr.push_back(std::move(child));
                ws();
                if (p < end && *p == ',')
                {
                    ++p;
                    continue;
                }
                if (p < end && *p == ']')
                {
                    ++p;
                    return true;
                }
                return fail("expected ',' or ']'");
            }
        }
        if (c == '"')
        {
            v.kind = Value::String;
            return string(v.str);
        }
        if (lit("true"))
        {
            v.kind = Value::Bool;
            v.b = true;
            return true;
        }
        if (lit("false"))
        {
            v.kind = Value::Bool;
            v.b = false;
            return true;
        }
        if (lit("null"))
        {
            v.kind = Value::Null;
            return true;
        }
        // number
        const char* s = p;
        if (p < end && (*p == '-' || *p == '+'))
            ++p;
        while (p < end && (std::isdigit(static_cast<unsigned char>(*p)) || *p == '.' || *p == 'e' || *p == 'E' ||
                           *p == '-' || *p == '+'))
            ++p;
        if (p == s)
            return fail("unexpected character");
        std::string num(s, p);
        char* e = nullptr;
        v.kind = Value::Number;
        v.num = std::strtod(num.c_str(), &e);
        if (!e || *e != '\0')
            return fail("bad number");
        return true;
    }
};

static bool parse(const char* text, Value& out, std::string& err)
{
    Parser ps{text, text + std::strlen(text), {}};
    if (!ps.value(out, 0))
    {
        err = ps.err;
        return false;
    }
    ps.ws();
    if (ps.p != ps.end)
    {
        err = "trailing characters";
        return false;
    }
    return true;
}

}  // namespace json

// Default ComputeSettings document: the key layout of the reference's ComputeSettings
// serialisation (version V1) with the reference's default values.
static const char* kDefaultComputeSettings = R"JSON({
 "version": "v1",
 "image_rendering": {
  "image_mode": "RAW", "batch_size": 1, "time_transformation_stride": 1,
  "filter2d": {"enabled": false, "inner_radius": 0, "outer_radius": 1},
  "space_transformation": "NONE", "time_transformation": "NONE", "time_transformation_size": 1,
  "lambda": 8.519999710188131e-07, "propagation_distance": 0.0,
  "convolution": {"type": "None", "divide": false},
  "input_filter": {"type": "None"}
 },
 "view": {
  "image_type": "MODULUS", "fft_shift": false,
  "x": {"width": 0, "start": 0}, "y": {"width": 0, "start": 0},
  "z": {"width": 0, "start": 0}, "z2": {"width": 0, "start": 0},
  "window": {
   "xy": {"log_enabled": false, "contrast": {"enabled": false, "auto_refresh": true, "invert": false, "min": 1.0, "max": 65535.0},
          "horizontal_flip": false, "rotation": 0.0, "output_image_accumulation": 1, "enabled": true},
   "yz": {"log_enabled": false, "contrast": {"enabled": false, "auto_refresh": true, "invert": false, "min": 1.0, "max": 65535.0},
          "horizontal_flip": false, "rotation": 0.0, "output_image_accumulation": 1, "enabled": false},
   "xz": {"log_enabled": false, "contrast": {"enabled": false, "auto_refresh": true, "invert": false, "min": 1.0, "max": 65535.0},
          "horizontal_flip": false, "rotation": 0.0, "output_image_accumulation": 1, "enabled": false},
   "filter2d": {"log_enabled": false, "contrast": {"enabled": false, "auto_refresh": true, "invert": false, "min": 1.0, "max": 65535.0}}
  },
  "renorm": true,
  "reticle": {"display_enabled": false, "scale": 0.5},
  "registration": {"registration_enabled": false, "registration_zone": 0.7}
 },
 "color_composite_image": {
  "mode": "RGB", "auto_weight": false,
  "rgb": {"frame_index": {"min": 0, "max": 0}, "weight": {"r": 1.0, "g": 1.0, "b": 1.0}},
  "hsv": {
   "h": {"frame_index": {"min": 0, "max": 0, "activated": false}, "slider_threshold": {"min": 0.01, "max": 1.0},
         "threshold": {"min": 0.2, "max": 99.8}, "slider_shift": {"min": 0.0, "max": 1.0}},
   "s": {"frame_index": {"min": 0, "max": 0, "activated": false}, "slider_threshold": {"min": 0.01, "max": 1.0},
         "threshold": {"min": 0.2, "max": 99.8}},
   "v": {"frame_index": {"min": 0, "max": 0, "activated": false}, "slider_threshold": {"min": 0.01, "max": 1.0},
         "threshold": {"min": 0.2, "max": 99.8}}
  }
 },
 "advanced": {
  "buffer_size": {"input": 512, "file": 1024, "record": 1024, "output": 1024, "time_transformation_cuts": 512},
  "filter2d_smooth": {"low": 0, "high": 1},
  "contrast": {"lower": 0.02, "upper": 99.98, "frame_index_offset": 2},
  "renorm_constant": 5, "raw_bitshift": 0, "nb_frames_to_record": 0
 }
})JSON";

static bool merge(json::Value& base, const json::Value& upd, std::string& err, const std::string& path)
{
    for (const auto& kv : upd.obj)
    {
        json::Value* b = base.find(kv.first);
        if (!b)
        {
            err = "key '" + path + kv.first + "' is not a compute setting";
            return false;
        }
        if (b->kind == json::Value::Object && kv.second.kind == json::Value::Object)
        {
            if (!merge(*b, kv.second, err, path + kv.first + "."))
                return false;
        }
        else
            *b = kv.second;
    }
    return true;
}

static const json::Value* at(const json::Value& root, std::initializer_list<const char*> path)
{
    const json::Value* v = &root;
    for (const char* k : path)
    {
        if (!v || v->kind != json::Value::Object)
            return nullptr;
        v = v->find(k);
    }
    return v;
}

static bool get_num(const json::Value& root, std::initializer_list<const char*> path, double& out)
{
    const json::Value* v = at(root, path);
    if (!v)
        return false;
    if (v->kind == json::Value::Number)
        out = v->num;
    else if (v->kind == json::Value::Bool)
        out = v->b ? 1.0 : 0.0;
    else
        return false;
    return true;
}

static bool get_str(const json::Value& root, std::initializer_list<const char*> path, std::string& out)
{
    const json::Value* v = at(root, path);
    if (!v || v->kind != json::Value::String)
        return false;
    out = v->str;
    return true;
}

int space_from_string(const std::string& s)
{
    if (s == "NONE" || s == "None")
        return HV_SPACE_NONE;
    if (s == "FRESNELTR" || s == "Fresnel Tr." || s == "FFT1" || s == "1FFT")
        return HV_SPACE_FRESNELTR;
    if (s == "ANGULARSP" || s == "Angular SP." || s == "FFT2" || s == "2FFT")
        return HV_SPACE_ANGULARSP;
    return -1;
}

int time_from_string(const std::string& s)
{
    if (s == "NONE" || s == "None")
        return HV_TIME_NONE;
    if (s == "STFT")
        return HV_TIME_STFT;
    if (s == "PCA")
        return HV_TIME_PCA;
    if (s == "SSA_STFT")
        return HV_TIME_SSA_STFT;
    return -1;
}

int img_from_string(const std::string& s)
{
    if (s == "MODULUS")
        return HV_IMG_MODULUS;
    if (s == "SQUARED_MODULUS")
        return HV_IMG_SQUARED_MODULUS;
    if (s == "ARGUMENT")
        return HV_IMG_ARGUMENT;
    if (s == "PHASE_INCREASE" || s == "COMPOSITE" || s == "MOMENTS_0" || s == "MOMENTS_1" || s == "MOMENTS_2")
        return 100;  // reference image types outside this path
    return -1;
}

void settings_default(hv_settings* s)
{
    std::memset(s, 0, sizeof(*s));
    s->space_transformation = HV_SPACE_NONE;
    s->time_transformation = HV_TIME_NONE;
    s->time_transformation_size = 1;
    s->time_stride = 1;
    s->batch_size = 1;
    s->lambda = 852e-9f;
    s->z_distance = 0.0f;
    s->pixel_size = 12.0f;
    s->image_type = HV_IMG_MODULUS;
    s->p_start = 0;
    s->p_width = 0;
    s->fft_shift = 0;
    s->renorm = 1;
    s->renorm_constant = 5;
    s->accumulation = 1;
    s->log_enabled = 0;
    s->contrast_enabled = 0;
    s->contrast_auto_refresh = 1;
    s->contrast_invert = 0;
    s->contrast_min = 1.0f;
    s->contrast_max = 65535.0f;
    s->contrast_lower = 0.02f;
    s->contrast_upper = 99.98f;
    s->reticle_display = 0;
    s->reticle_scale = 0.5f;
    s->unwrap_2d = 0;
    s->lens_mode = HV_LENS_FP64;
    s->output_buffer_size = 1024;
    s->input_buffer_size = 512;
}

hv_status settings_from_json(const char* text, hv_settings* s)
{
    if (!text || !s)
        return HV_INVALID_VALUE;
    json::Value doc, base;
    std::string err;
    if (!json::parse(text, doc, err))
    {
        set_last_error_msg(("invalid json: " + err).c_str());
        return HV_FAILURE;
    }
    if (doc.kind != json::Value::Object || doc.obj.empty())
    {
        set_last_error_msg("empty compute settings");
        return HV_NO_IN_DATA;
    }
    json::parse(kDefaultComputeSettings, base, err);
    // seed the base with the caller's current settings so a partial document keeps them
    if (!merge(base, doc, err, ""))
    {
        set_last_error_msg(err.c_str());
        return HV_FAILURE;
    }
    hv_settings out = *s;
    std::string str;
    double d;
    auto has = [&](std::initializer_list<const char*> p) { return at(doc, p) != nullptr; };
    if (has({"image_rendering", "space_transformation"}) && get_str(base, {"image_rendering", "space_transformation"}, str))
    {
        const int v = space_from_string(str);
        if (v < 0)
        {
            set_last_error_msg("unknown space_transformation");
            return HV_INVALID_VALUE;
        }
        out.space_transformation = v;
    }
    if (has({"image_rendering", "time_transformation"}) && get_str(base, {"image_rendering", "time_transformation"}, str))
    {
        const int v = time_from_string(str);
        if (v < 0)
        {
            set_last_error_msg("unknown time_transformation");
            return HV_INVALID_VALUE;
        }
        out.time_transformation = v;
    }
    if (has({"view", "image_type"}) && get_str(base, {"view", "image_type"}, str))
    {
        const int v = img_from_string(str);
        if (v < 0)
        {
            set_last_error_msg("unknown image_type");
            return HV_INVALID_VALUE;
        }
        out.image_type = v;
    }
    struct NumField
    {
        std::initializer_list<const char*> path;
        int kind;  // 0 int32, 1 float, 2 bool
        void* dst;
    };
    const NumField fields[] = {
        {{"image_rendering", "time_transformation_size"}, 0, &out.time_transformation_size},
        {{"image_rendering", "time_transformation_stride"}, 0, &out.time_stride},
        {{"image_rendering", "batch_size"}, 0, &out.batch_size},
        {{"image_rendering", "lambda"}, 1, &out.lambda},
        {{"image_rendering", "propagation_distance"}, 1, &out.z_distance},
        {{"view", "fft_shift"}, 2, &out.fft_shift},
        {{"view", "renorm"}, 2, &out.renorm},
        {{"view", "z", "start"}, 0, &out.p_start},
        {{"view", "z", "width"}, 0, &out.p_width},
        {{"view", "window", "xy", "output_image_accumulation"}, 0, &out.accumulation},
        {{"view", "window", "xy", "log_enabled"}, 2, &out.log_enabled},
        {{"view", "window", "xy", "contrast", "enabled"}, 2, &out.contrast_enabled},
        {{"view", "window", "xy", "contrast", "auto_refresh"}, 2, &out.contrast_auto_refresh},
        {{"view", "window", "xy", "contrast", "invert"}, 2, &out.contrast_invert},
        {{"view", "window", "xy", "contrast", "min"}, 1, &out.contrast_min},
        {{"view", "window", "xy", "contrast", "max"}, 1, &out.contrast_max},
        {{"view", "reticle", "display_enabled"}, 2, &out.reticle_display},
        {{"view", "reticle", "scale"}, 1, &out.reticle_scale},
        {{"advanced", "contrast", "lower"}, 1, &out.contrast_lower},
        {{"advanced", "contrast", "upper"}, 1, &out.contrast_upper},
        {{"advanced", "renorm_constant"}, 0, &out.renorm_constant},
        {{"advanced", "buffer_size", "output"}, 0, &out.output_buffer_size},
        {{"advanced", "buffer_size", "input"}, 0, &out.input_buffer_size},
    };
    for (const auto& f : fields)
    {
        if (!at(doc, f.path))
            continue;
        if (!get_num(base, f.path, d))
        {
            set_last_error_msg("compute setting has the wrong type");
            return HV_FAILURE;
        }
        if (f.kind == 0)
            *static_cast<int32_t*>(f.dst) = static_cast<int32_t>(d);
        else if (f.kind == 1)
            *static_cast<float*>(f.dst) = static_cast<float>(d);
        else
            *static_cast<int32_t*>(f.dst) = d != 0.0 ? 1 : 0;
    }
    if (has({"image_rendering", "image_mode"}) && get_str(base, {"image_rendering", "image_mode"}, str))
    {
        if (str != "HOLOGRAM" && str != "RAW")
        {
            set_last_error_msg("unknown image_mode");
            return HV_INVALID_VALUE;
        }
    }
    *s = out;
    return HV_OK;
}

hv_status settings_validate(hv_settings* s, const hv_frame_desc* fd)
{
    if (!s)
        return HV_INVALID_VALUE;
    if (s->batch_size < 1)
        s->batch_size = 1;
    if (s->input_buffer_size > 0 && s->batch_size > s->input_buffer_size)
        s->batch_size = s->input_buffer_size;  // set_batch_size (transform_api.cc:25-30)
    // set_time_stride (transform_api.cc:49-70): >= batch and a multiple of it
    if (s->time_stride < s->batch_size)
        s->time_stride = s->batch_size;
    if (s->time_stride % s->batch_size != 0)
        s->time_stride -= s->time_stride % s->batch_size;
    if (s->time_transformation_size < 1)
        s->time_transformation_size = 1;
    if (s->lambda < 0.f)
        s->lambda = 0.f;
    if (s->z_distance == 0.f)
        s->z_distance = 0.000001f;  // set_z_distance (transform_api.cc:109-120)
    // check_p_limits (transform_api.cc:170-186)
    const int T = s->time_transformation_size;
    int upper = T - 1;
    if (s->p_width > upper)
        s->p_width = upper;
    if (s->p_width < 0)
        s->p_width = 0;
    upper -= s->p_width;
    if (s->p_start > upper)
        s->p_start = upper;
    if (s->p_start < 0)
        s->p_start = 0;
    if (s->accumulation < 0)
        s->accumulation = 0;
    if (s->output_buffer_size < 1)
        s->output_buffer_size = 1;
    if (s->image_type != HV_IMG_MODULUS && s->image_type != HV_IMG_SQUARED_MODULUS && s->image_type != HV_IMG_ARGUMENT)
    {
        set_last_error_msg("image type outside the hologram path (modulus, squared modulus, argument)");
        return HV_WRONG_IMG_TYPE;
    }
    if (s->time_transformation == HV_TIME_SSA_STFT)
    {
        set_last_error_msg("SSA_STFT is not implemented");
        return HV_ERR_UNSUPPORTED;
    }
    if (fd)
    {
        if (fd->width == 0 || fd->height == 0)
            return HV_INVALID_VALUE;
        if (fd->depth != 1 && fd->depth != 2 && fd->depth != 4)
        {
            set_last_error_msg("pixel depth must be 1, 2 or 4 bytes");
            return HV_INVALID_VALUE;
        }
        if (s->space_transformation != HV_SPACE_NONE &&
            (!fft_size_supported(fd->width) || !fft_size_supported(fd->height)))
        {
            set_last_error_msg("frame size not supported by the shared-memory FFT");
            return HV_ERR_UNSUPPORTED;
        }
        if (s->fft_shift && ((fd->width & 1) || (fd->height & 1)))
        {
            set_last_error_msg("fftshift needs even width and height");
            return HV_INVALID_VALUE;
        }
        if (s->unwrap_2d && s->image_type == HV_IMG_ARGUMENT &&
            (!fft_size_supported(fd->width) || !fft_size_supported(fd->height)))
        {
            set_last_error_msg("frame size not supported by the unwrap FFT");
            return HV_ERR_UNSUPPORTED;
        }
    }
    return HV_OK;
}

}  // namespace hv
