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
#include "json_lite.h"
#include "settings_internal.h"

namespace hv {

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

// lenient: keys absent from the default document are skipped instead of refused (.holo footers
// written by other versions carry settings this build does not use)
static bool merge(json::Value& base, const json::Value& upd, std::string& err, const std::string& path,
                  bool lenient = false)
{
    for (const auto& kv : upd.obj)
    {
        json::Value* b = base.find(kv.first);
        if (!b)
        {
            if (lenient)
                continue;
            err = "key '" + path + kv.first + "' is not a compute setting";
            return false;
        }
        if (b->kind == json::Value::Object && kv.second.kind == json::Value::Object)
        {
            if (!merge(*b, kv.second, err, path + kv.first + ".", lenient))
                return false;
        }
        else if (b->kind == json::Value::Object || kv.second.kind == json::Value::Object)
        {
            if (lenient)
                continue;
            err = "key '" + path + kv.first + "' has the wrong type";
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
    if (s == "PHASE_INCREASE")
        return HV_IMG_PHASE_INCREASE;
    if (s == "MOMENTS_0")
        return HV_IMG_MOMENTS_0;
    if (s == "MOMENTS_1")
        return HV_IMG_MOMENTS_1;
    if (s == "MOMENTS_2")
        return HV_IMG_MOMENTS_2;
    if (s == "COMPOSITE")
        return 100;  // reference image type outside this path
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
    s->camera_fps = 0;  // settings::CameraFps{0} (holovibes.hh:446)
    s->q_start = 0;
    s->q_width = 0;
    // Filter2dN1{0}, Filter2dN2{1}, Filter2dSmoothLow{0}, Filter2dSmoothHigh{1} (holovibes.hh:405-408)
    s->filter2d_enabled = 0;
    s->filter2d_n1 = 0;
    s->filter2d_n2 = 1;
    s->filter2d_smooth_low = 0;
    s->filter2d_smooth_high = 1;
    // XZ / YZ windows: View_XZ / View_YZ defaults (view_struct.hh), CutsContrastPOffset{2},
    // TimeTransformationCutsOutputBufferSize{512}
    s->cuts_enabled = 0;
    s->x_start = s->x_width = s->y_start = s->y_width = 0;
    s->xz_accumulation = s->yz_accumulation = 1;
    s->xz_log_enabled = s->yz_log_enabled = 0;
    s->xz_contrast_enabled = s->yz_contrast_enabled = 0;
    s->xz_contrast_auto_refresh = s->yz_contrast_auto_refresh = 1;
    s->xz_contrast_invert = s->yz_contrast_invert = 0;
    s->xz_contrast_min = s->yz_contrast_min = 1.0f;
    s->xz_contrast_max = s->yz_contrast_max = 65535.0f;
    s->cuts_contrast_offset = 2;
    s->cuts_buffer_size = 512;
    // filter2D view window: View_Window defaults (view_struct.hh)
    s->filter2d_view_enabled = 0;
    s->filter2d_log_enabled = 0;
    s->filter2d_contrast_enabled = 0;
    s->filter2d_contrast_auto_refresh = 1;
    s->filter2d_contrast_invert = 0;
    s->filter2d_contrast_min = 1.0f;
    s->filter2d_contrast_max = 65535.0f;
}

hv_status settings_from_json(const char* text, hv_settings* s)
{
    if (!text || !s)
        return HV_INVALID_VALUE;
    json::Value doc;
    std::string err;
    if (!json::parse(text, doc, err))
    {
        set_last_error_msg(("invalid json: " + err).c_str());
        return HV_FAILURE;
    }
    return settings_from_value(doc, s, false);
}

hv_status settings_from_value(const json::Value& doc, hv_settings* s, bool lenient)
{
    json::Value base;
    std::string err;
    if (doc.kind != json::Value::Object || doc.obj.empty())
    {
        set_last_error_msg("empty compute settings");
        return HV_NO_IN_DATA;
    }
    json::parse(kDefaultComputeSettings, base, err);
    // seed the base with the caller's current settings so a partial document keeps them
    if (!merge(base, doc, err, "", lenient))
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
        {{"view", "z2", "start"}, 0, &out.q_start},
        {{"view", "z2", "width"}, 0, &out.q_width},
        {{"image_rendering", "filter2d", "enabled"}, 2, &out.filter2d_enabled},
        {{"image_rendering", "filter2d", "inner_radius"}, 0, &out.filter2d_n1},
        {{"image_rendering", "filter2d", "outer_radius"}, 0, &out.filter2d_n2},
        {{"advanced", "filter2d_smooth", "low"}, 0, &out.filter2d_smooth_low},
        {{"advanced", "filter2d_smooth", "high"}, 0, &out.filter2d_smooth_high},
        {{"view", "x", "start"}, 0, &out.x_start},
        {{"view", "x", "width"}, 0, &out.x_width},
        {{"view", "y", "start"}, 0, &out.y_start},
        {{"view", "y", "width"}, 0, &out.y_width},
        {{"view", "window", "xz", "output_image_accumulation"}, 0, &out.xz_accumulation},
        {{"view", "window", "yz", "output_image_accumulation"}, 0, &out.yz_accumulation},
        {{"view", "window", "xz", "log_enabled"}, 2, &out.xz_log_enabled},
        {{"view", "window", "yz", "log_enabled"}, 2, &out.yz_log_enabled},
        {{"view", "window", "xz", "contrast", "enabled"}, 2, &out.xz_contrast_enabled},
        {{"view", "window", "xz", "contrast", "auto_refresh"}, 2, &out.xz_contrast_auto_refresh},
        {{"view", "window", "xz", "contrast", "invert"}, 2, &out.xz_contrast_invert},
        {{"view", "window", "xz", "contrast", "min"}, 1, &out.xz_contrast_min},
        {{"view", "window", "xz", "contrast", "max"}, 1, &out.xz_contrast_max},
        {{"view", "window", "yz", "contrast", "enabled"}, 2, &out.yz_contrast_enabled},
        {{"view", "window", "yz", "contrast", "auto_refresh"}, 2, &out.yz_contrast_auto_refresh},
        {{"view", "window", "yz", "contrast", "invert"}, 2, &out.yz_contrast_invert},
        {{"view", "window", "yz", "contrast", "min"}, 1, &out.yz_contrast_min},
        {{"view", "window", "yz", "contrast", "max"}, 1, &out.yz_contrast_max},
        {{"advanced", "contrast", "frame_index_offset"}, 0, &out.cuts_contrast_offset},
        {{"advanced", "buffer_size", "time_transformation_cuts"}, 0, &out.cuts_buffer_size},
        {{"view", "window", "filter2d", "log_enabled"}, 2, &out.filter2d_log_enabled},
        {{"view", "window", "filter2d", "contrast", "enabled"}, 2, &out.filter2d_contrast_enabled},
        {{"view", "window", "filter2d", "contrast", "auto_refresh"}, 2, &out.filter2d_contrast_auto_refresh},
        {{"view", "window", "filter2d", "contrast", "invert"}, 2, &out.filter2d_contrast_invert},
        {{"view", "window", "filter2d", "contrast", "min"}, 1, &out.filter2d_contrast_min},
        {{"view", "window", "filter2d", "contrast", "max"}, 1, &out.filter2d_contrast_max},
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


// ------------------------------------------------------------------------------ serialisation
static json::Value* ensure(json::Value& root, std::initializer_list<const char*> path)
{
    json::Value* v = &root;
    for (const char* k : path)
    {
        if (v->kind != json::Value::Object)
        {
            *v = json::Value{};
            v->kind = json::Value::Object;
        }
        json::Value* c = v->find(k);
        if (!c)
        {
            v->obj.emplace_back(k, json::Value{});
            c = &v->obj.back().second;
        }
        v = c;
    }
    return v;
}

static void set_num(json::Value& root, std::initializer_list<const char*> path, double x)
{
    json::Value* v = ensure(root, path);
    *v = json::Value{};
    v->kind = json::Value::Number;
    v->num = x;
}

static void set_bool(json::Value& root, std::initializer_list<const char*> path, bool b)
{
    json::Value* v = ensure(root, path);
    *v = json::Value{};
    v->kind = json::Value::Bool;
    v->b = b;
}

static void set_str(json::Value& root, std::initializer_list<const char*> path, const char* x)
{
    json::Value* v = ensure(root, path);
    *v = json::Value{};
    v->kind = json::Value::String;
    v->str = x;
}

// The compute-settings document (current layout, version v1) of a settings record: the default
// document with every field this build reads set from `s` (ComputeSettingsApi::
// compute_settings_to_json, compute_settings.cc:38-99, for the keys of this path).
void settings_to_value(const hv_settings* s, json::Value& doc)
{
    std::string err;
    doc = json::Value{};
    json::parse(kDefaultComputeSettings, doc, err);
    static const char* space[] = {"NONE", "FRESNELTR", "ANGULARSP"};
    static const char* time[] = {"NONE", "STFT", "PCA", "SSA_STFT"};
    static const char* img[] = {"MODULUS", "SQUARED_MODULUS", "ARGUMENT", "PHASE_INCREASE", "COMPOSITE",
                                "MOMENTS_0", "MOMENTS_1", "MOMENTS_2"};
    set_str(doc, {"image_rendering", "image_mode"}, "HOLOGRAM");
    set_str(doc, {"image_rendering", "space_transformation"},
            space[s->space_transformation >= 0 && s->space_transformation <= 2 ? s->space_transformation : 0]);
    set_str(doc, {"image_rendering", "time_transformation"},
            time[s->time_transformation >= 0 && s->time_transformation <= 3 ? s->time_transformation : 0]);
    set_num(doc, {"image_rendering", "time_transformation_size"}, s->time_transformation_size);
    set_num(doc, {"image_rendering", "time_transformation_stride"}, s->time_stride);
    set_num(doc, {"image_rendering", "batch_size"}, s->batch_size);
    set_num(doc, {"image_rendering", "lambda"}, s->lambda);
    set_num(doc, {"image_rendering", "propagation_distance"}, s->z_distance);
    set_str(doc, {"view", "image_type"}, img[s->image_type >= 0 && s->image_type <= 7 ? s->image_type : 0]);
    set_bool(doc, {"view", "fft_shift"}, s->fft_shift != 0);
    set_bool(doc, {"view", "renorm"}, s->renorm != 0);
    set_num(doc, {"view", "z", "start"}, s->p_start);
    set_num(doc, {"view", "z", "width"}, s->p_width);
    set_num(doc, {"view", "z2", "start"}, s->q_start);
    set_num(doc, {"view", "z2", "width"}, s->q_width);
    set_bool(doc, {"image_rendering", "filter2d", "enabled"}, s->filter2d_enabled != 0);
    set_num(doc, {"image_rendering", "filter2d", "inner_radius"}, s->filter2d_n1);
    set_num(doc, {"image_rendering", "filter2d", "outer_radius"}, s->filter2d_n2);
    set_num(doc, {"advanced", "filter2d_smooth", "low"}, s->filter2d_smooth_low);
    set_num(doc, {"advanced", "filter2d_smooth", "high"}, s->filter2d_smooth_high);
    set_num(doc, {"view", "x", "start"}, s->x_start);
    set_num(doc, {"view", "x", "width"}, s->x_width);
    set_num(doc, {"view", "y", "start"}, s->y_start);
    set_num(doc, {"view", "y", "width"}, s->y_width);
    for (int w = 0; w < 2; ++w)
    {
        const char* win = w == 0 ? "xz" : "yz";
        set_num(doc, {"view", "window", win, "output_image_accumulation"}, w == 0 ? s->xz_accumulation : s->yz_accumulation);
        set_bool(doc, {"view", "window", win, "log_enabled"}, (w == 0 ? s->xz_log_enabled : s->yz_log_enabled) != 0);
        set_bool(doc, {"view", "window", win, "contrast", "enabled"},
                 (w == 0 ? s->xz_contrast_enabled : s->yz_contrast_enabled) != 0);
        set_bool(doc, {"view", "window", win, "contrast", "auto_refresh"},
                 (w == 0 ? s->xz_contrast_auto_refresh : s->yz_contrast_auto_refresh) != 0);
        set_bool(doc, {"view", "window", win, "contrast", "invert"},
                 (w == 0 ? s->xz_contrast_invert : s->yz_contrast_invert) != 0);
        set_num(doc, {"view", "window", win, "contrast", "min"}, w == 0 ? s->xz_contrast_min : s->yz_contrast_min);
        set_num(doc, {"view", "window", win, "contrast", "max"}, w == 0 ? s->xz_contrast_max : s->yz_contrast_max);
    }
    set_num(doc, {"advanced", "contrast", "frame_index_offset"}, s->cuts_contrast_offset);
    set_num(doc, {"advanced", "buffer_size", "time_transformation_cuts"}, s->cuts_buffer_size);
    set_bool(doc, {"view", "window", "filter2d", "log_enabled"}, s->filter2d_log_enabled != 0);
    set_bool(doc, {"view", "window", "filter2d", "contrast", "enabled"}, s->filter2d_contrast_enabled != 0);
    set_bool(doc, {"view", "window", "filter2d", "contrast", "auto_refresh"}, s->filter2d_contrast_auto_refresh != 0);
    set_bool(doc, {"view", "window", "filter2d", "contrast", "invert"}, s->filter2d_contrast_invert != 0);
    set_num(doc, {"view", "window", "filter2d", "contrast", "min"}, s->filter2d_contrast_min);
    set_num(doc, {"view", "window", "filter2d", "contrast", "max"}, s->filter2d_contrast_max);
    set_num(doc, {"view", "window", "xy", "output_image_accumulation"}, s->accumulation);
    set_bool(doc, {"view", "window", "xy", "log_enabled"}, s->log_enabled != 0);
    set_bool(doc, {"view", "window", "xy", "contrast", "enabled"}, s->contrast_enabled != 0);
    set_bool(doc, {"view", "window", "xy", "contrast", "auto_refresh"}, s->contrast_auto_refresh != 0);
    set_bool(doc, {"view", "window", "xy", "contrast", "invert"}, s->contrast_invert != 0);
    set_num(doc, {"view", "window", "xy", "contrast", "min"}, s->contrast_min);
    set_num(doc, {"view", "window", "xy", "contrast", "max"}, s->contrast_max);
    set_bool(doc, {"view", "reticle", "display_enabled"}, s->reticle_display != 0);
    set_num(doc, {"view", "reticle", "scale"}, s->reticle_scale);
    set_num(doc, {"advanced", "contrast", "lower"}, s->contrast_lower);
    set_num(doc, {"advanced", "contrast", "upper"}, s->contrast_upper);
    set_num(doc, {"advanced", "renorm_constant"}, s->renorm_constant);
    set_num(doc, {"advanced", "buffer_size", "output"}, s->output_buffer_size);
    set_num(doc, {"advanced", "buffer_size", "input"}, s->input_buffer_size);
}

// Compute-settings documents without a "version" key are version v0: v1 dropped three keys and
// added the version tag and the registration block (ComputeSettingsConverter,
// compute_settings_converter.cc:8-100 with its patch table assets/json_patches_settings). Returns
// false for an unknown version.
bool settings_convert_to_current(json::Value& doc)
{
    if (doc.kind != json::Value::Object)
        return false;
    const json::Value* ver = doc.find("version");
    if (ver)
        return ver->kind == json::Value::String && ver->str == "v1";
    auto drop = [&](std::initializer_list<const char*> path) {
        json::Value* v = &doc;
        const char* last = nullptr;
        json::Value* parent = nullptr;
        for (const char* k : path)
        {
            if (!v || v->kind != json::Value::Object)
                return;
            parent = v;
            last = k;
            v = v->find(k);
        }
        if (!v || !parent)
            return;
        for (size_t i = 0; i < parent->obj.size(); ++i)
            if (parent->obj[i].first == last)
            {
                parent->obj.erase(parent->obj.begin() + static_cast<std::ptrdiff_t>(i));
                return;
            }
    };
    drop({"image_rendering", "input_filter", "enabled"});
    drop({"image_rendering", "convolution", "enabled"});
    drop({"advanced", "record_mode"});
    set_str(doc, {"version"}, "v1");
    set_bool(doc, {"view", "registration", "registration_enabled"}, false);
    set_num(doc, {"view", "registration", "registration_zone"}, 0.7);
    return true;
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
    // check_q_limits (transform_api.cc:208-225)
    upper = T - 1;
    if (s->q_width > upper)
        s->q_width = upper;
    if (s->q_width < 0)
        s->q_width = 0;
    upper -= s->q_width;
    if (s->q_start > upper)
        s->q_start = upper;
    if (s->q_start < 0)
        s->q_start = 0;
    if (s->accumulation < 0)
        s->accumulation = 0;
    if (s->output_buffer_size < 1)
        s->output_buffer_size = 1;
    if (s->image_type < HV_IMG_MODULUS || s->image_type > HV_IMG_MOMENTS_2 || s->image_type == 4)
    {
        set_last_error_msg("image type outside the hologram path (composite or unknown)");
        return HV_WRONG_IMG_TYPE;
    }
    if (s->camera_fps < 0)
        s->camera_fps = 0;
    if (s->xz_accumulation < 0)
        s->xz_accumulation = 0;
    if (s->yz_accumulation < 0)
        s->yz_accumulation = 0;
    if (s->cuts_contrast_offset < 0)
        s->cuts_contrast_offset = 0;
    if (s->cuts_buffer_size < 1)
        s->cuts_buffer_size = 1;
    if (s->cuts_enabled && !cuts_supported(s->time_transformation_size))
    {
        set_last_error_msg("time cuts: time window above 512 frames");
        return HV_ERR_UNSUPPORTED;
    }
    // Filter2dApi::set_filter2d_n1 / n2 (filter2d_api.cc:27-63): 0 <= n1 < n2
    if (s->filter2d_enabled && (s->filter2d_n1 < 0 || s->filter2d_n2 <= s->filter2d_n1 ||
                                s->filter2d_smooth_low < 0 || s->filter2d_smooth_high < 0))
    {
        set_last_error_msg("filter2d radii must satisfy 0 <= inner < outer, smoothing >= 0");
        return HV_INVALID_VALUE;
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
        // the cursor band must stay inside the frame (fill_32bit_slices reads x + y W up to xmax,
        // ymax); a cursor outside the frame leaves the cuts as they are (fourier_transform.cc:484)
        if (s->cuts_enabled && (s->x_width < 0 || s->y_width < 0 || s->x_start < 0 || s->y_start < 0 ||
                                (s->x_start < static_cast<int>(fd->width) &&
                                 s->x_start + s->x_width >= static_cast<int>(fd->width)) ||
                                (s->y_start < static_cast<int>(fd->height) &&
                                 s->y_start + s->y_width >= static_cast<int>(fd->height))))
        {
            set_last_error_msg("time cuts: cursor band outside the frame");
            return HV_INVALID_VALUE;
        }
        if (s->filter2d_enabled)
        {
            if ((fd->width & 1) || (fd->height & 1))
            {
                set_last_error_msg("filter2d needs even width and height (shifted mask)");
                return HV_INVALID_VALUE;
            }
            if (!fft_size_supported(fd->width) || !fft_size_supported(fd->height))
            {
                set_last_error_msg("frame size not supported by the shared-memory FFT");
                return HV_ERR_UNSUPPORTED;
            }
        }
        if (s->unwrap_2d && (s->image_type == HV_IMG_ARGUMENT || s->image_type == HV_IMG_PHASE_INCREASE) &&
            (!fft_size_supported(fd->width) || !fft_size_supported(fd->height)))
        {
            set_last_error_msg("frame size not supported by the unwrap FFT");
            return HV_ERR_UNSUPPORTED;
        }
    }
    return HV_OK;
}

}  // namespace hv
