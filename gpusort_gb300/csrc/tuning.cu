// Tuning table of a context (gs_ctx_set_tuning, gs_ctx_load_tuning,
// gs_ctx_choice): which pass tile shape and how many SampleSort buckets a
// call of a given key type, payload width and size uses, and the JSON file
// the autotuner writes.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "context.h"

namespace gs {

namespace {

uint32_t floor_log2(uint64_t n) { return n ? 63u - uint32_t(__builtin_clzll(n)) : 0u; }

// First tuning entry for (key width and kind, payload width, size).
const gs_tuning_entry* find_tuning(const gs_ctx* ctx, int kb, uint32_t kk, int vb, uint64_t n) {
  const uint32_t lg = floor_log2(n);
  for (const gs_tuning_entry& e : ctx->tuning) {
    int ekb = 0;
    uint32_t ekk = 0;
    if (!dtype_info(gs_dtype(e.key_dtype), &ekb, &ekk) || ekb != kb || ekk != kk) continue;
    if (e.val_bytes != vb || lg < e.log2n_min || lg > e.log2n_max) continue;
    return &e;
  }
  return nullptr;
}

}  // namespace

int pass_shape_for(const gs_ctx* ctx, int kb, uint32_t kk, int vb, uint64_t n) {
  if (ctx->shape >= 0) return ctx->shape;
  const gs_tuning_entry* e = find_tuning(ctx, kb, kk, vb, n);
  if (e && e->pass_shape >= 0) return e->pass_shape;
  return gs::radix_default_shape(kb, vb, n);
}

uint32_t partitions_for(const gs_ctx* ctx, int kb, uint32_t kk, uint64_t n, const gs_opts* o) {
  if (o && o->partitions) return o->partitions;
  const gs_tuning_entry* e = find_tuning(ctx, kb, kk, 0, n);
  if (e && e->partitions) return e->partitions;
  return 64;
}

namespace {

bool entry_valid(const gs_tuning_entry& e) {
  int kb = 0;
  uint32_t kk = 0;
  return dtype_info(gs_dtype(e.key_dtype), &kb, &kk) &&
         (e.val_bytes == 0 || e.val_bytes == 4 || e.val_bytes == 8) &&
         e.log2n_min <= e.log2n_max && e.log2n_max <= 63 && e.pass_shape >= -1 &&
         e.pass_shape < gs::radix_num_shapes() && e.partitions <= gs::RADIX &&
         (e.partitions == 0 || e.partitions >= 2);
}

// Minimal JSON reader for the tuning file: any object holding "key_dtype"
// (at any depth) is an entry; other keys and values are skipped.
struct Json {
  const char* p;
  const char* e;
  std::vector<gs_tuning_entry>* out;
  bool ok = true;

  void ws() {
    while (p < e && (*p == ' ' || *p == '\n' || *p == '\r' || *p == '\t')) ++p;
  }
  bool lit(const char* w) {
    const size_t k = std::strlen(w);
    if (size_t(e - p) < k || std::strncmp(p, w, k) != 0) return false;
    p += k;
    return true;
  }
  bool str(std::string* s) {
    if (p >= e || *p != '"') return false;
    ++p;
    while (p < e && *p != '"') {
      if (*p == '\\') {
        if (++p >= e) return false;
      }
      if (s) s->push_back(*p);
      ++p;
    }
    if (p >= e) return false;
    ++p;
    return true;
  }
  bool num(double* v) {
    char* end = nullptr;
    const double x = std::strtod(p, &end);
    if (end == p || end > e) return false;
    p = end;
    if (v) *v = x;
    return true;
  }
  // value; scalars are reported through *is_num / *d / *s
  bool value(bool* is_num, double* d, std::string* s, int depth) {
    if (depth > 32) return false;
    ws();
    if (p >= e) return false;
    if (*p == '{') return object(depth + 1);
    if (*p == '[') {
      ++p;
      ws();
      if (p < e && *p == ']') { ++p; return true; }
      while (true) {
        if (!value(nullptr, nullptr, nullptr, depth + 1)) return false;
        ws();
        if (p < e && *p == ',') { ++p; continue; }
        if (p < e && *p == ']') { ++p; return true; }
        return false;
      }
    }
    if (*p == '"') {
      if (is_num) *is_num = false;
      return str(s);
    }
    if (lit("true") || lit("false") || lit("null")) {
      if (is_num) *is_num = false;
      return true;
    }
    if (is_num) *is_num = true;
    return num(d);
  }
  bool object(int depth) {
    ++p;  // '{'
    gs_tuning_entry en{-1, 0, 0, 63, -1, 0};
    bool is_entry = false, bad = false;
    ws();
    if (p < e && *p == '}') { ++p; return true; }
    while (true) {
      ws();
      std::string key;
      if (!str(&key)) return false;
      ws();
      if (p >= e || *p != ':') return false;
      ++p;
      bool isn = false;
      double d = 0;
      std::string sv;
      if (!value(&isn, &d, &sv, depth)) return false;
      auto as_int = [&](int64_t lo, int64_t hi, int64_t* o) {
        if (!isn || d != double(int64_t(d)) || d < double(lo) || d > double(hi)) { bad = true; return; }
        *o = int64_t(d);
      };
      int64_t v = 0;
      if (key == "key_dtype") {
        is_entry = true;
        static const char* names[] = {"u32", "i32", "f32", "u64", "i64", "f64"};
        if (isn) { as_int(0, 5, &v); en.key_dtype = int32_t(v); }
        else {
          en.key_dtype = -1;
          for (int i = 0; i < 6; ++i) if (sv == names[i]) en.key_dtype = i;
          if (en.key_dtype < 0) bad = true;
        }
      } else if (key == "val_bytes") { as_int(0, 8, &v); en.val_bytes = int32_t(v); }
      else if (key == "log2n_min") { as_int(0, 63, &v); en.log2n_min = uint32_t(v); }
      else if (key == "log2n_max") { as_int(0, 63, &v); en.log2n_max = uint32_t(v); }
      else if (key == "pass_shape") { as_int(-1, 1 << 20, &v); en.pass_shape = int32_t(v); }
      else if (key == "partitions") { as_int(0, 1 << 20, &v); en.partitions = uint32_t(v); }
      ws();
      if (p < e && *p == ',') { ++p; continue; }
      if (p < e && *p == '}') { ++p; break; }
      return false;
    }
    if (is_entry) {
      if (bad || !entry_valid(en)) ok = false;
      else out->push_back(en);
    }
    return true;
  }
};

int parse_tuning(const char* json, std::vector<gs_tuning_entry>* out) {
  if (!json) return -1;
  Json j{json, json + std::strlen(json), out};
  if (!j.value(nullptr, nullptr, nullptr, 0)) return -1;
  j.ws();
  if (j.p != j.e || !j.ok) return -1;
  return int(out->size());
}

}  // namespace

}  // namespace gs

using namespace gs;

extern "C" {

gs_status gs_ctx_set_tuning(gs_ctx* ctx, const gs_tuning_entry* entries, uint32_t count) {
  if (!ctx) return fail(nullptr, GS_ERR_INVALID, "null context");
  if (count && !entries) return fail(ctx, GS_ERR_INVALID, "null tuning entries");
  for (uint32_t i = 0; i < count; ++i)
    if (!entry_valid(entries[i])) return fail(ctx, GS_ERR_INVALID, "invalid tuning entry");
  std::lock_guard<std::mutex> lock(ctx->mu);
  ctx->tuning.assign(entries, entries + count);
  return GS_OK;
}

int gs_tuning_parse(const char* json, gs_tuning_entry* out, uint32_t capacity) {
  std::vector<gs_tuning_entry> v;
  const int k = parse_tuning(json, &v);
  if (k < 0) return -1;
  if (out && uint32_t(k) <= capacity) std::copy(v.begin(), v.end(), out);
  return k;
}

gs_status gs_ctx_load_tuning(gs_ctx* ctx, const char* path) {
  if (!ctx || !path) return fail(ctx, GS_ERR_INVALID, "null context or path");
  FILE* f = std::fopen(path, "rb");
  if (!f) return fail(ctx, GS_ERR_INVALID, std::string("cannot open tuning file ") + path);
  std::string text;
  char buf[4096];
  size_t k;
  while ((k = std::fread(buf, 1, sizeof buf, f)) > 0) text.append(buf, k);
  std::fclose(f);
  std::vector<gs_tuning_entry> v;
  if (parse_tuning(text.c_str(), &v) < 0)
    return fail(ctx, GS_ERR_INVALID, std::string("malformed tuning file ") + path);
  std::lock_guard<std::mutex> lock(ctx->mu);
  ctx->tuning = std::move(v);
  return GS_OK;
}

gs_status gs_ctx_choice(gs_ctx* ctx, gs_dtype key_dtype, int val_bytes, uint64_t n,
                        int* pass_shape, uint32_t* partitions) {
  if (!ctx) return fail(nullptr, GS_ERR_INVALID, "null context");
  int kb = 0;
  uint32_t kk = 0;
  if (!dtype_info(key_dtype, &kb, &kk)) return fail(ctx, GS_ERR_BAD_DTYPE, "unknown key dtype");
  if (val_bytes != 0 && val_bytes != 4 && val_bytes != 8)
    return fail(ctx, GS_ERR_INVALID, "payload width must be 0, 4 or 8");
  std::lock_guard<std::mutex> lock(ctx->mu);
  if (pass_shape) *pass_shape = pass_shape_for(ctx, kb, kk, val_bytes, n);
  if (partitions) *partitions = partitions_for(ctx, kb, kk, n, nullptr);
  return GS_OK;
}

}  // extern "C"
