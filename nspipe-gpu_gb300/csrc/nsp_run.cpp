// nsp_run.cpp -- the time-integration driver of the C ABI (nsp_run_*, nsp_checkpoint_info,
// nsp_output_schedule): the reference's integrate() loop (mod_integrate.cu:98-160) with
// its time accumulators and output cadence (:109, :131-152), the diagnostic files of
// setIO / wrt_frc / wrt_qcr / wrt_ucr / wrt_mpr (mod_io_nonlinear.cu:260-318, 460-687),
// the final state dump (main.cu:42-44), and checkpoints with a JSON sidecar.
//
// Host code only: the context is driven through its public entry points (nsp_step in
// chunks that end where a row or a checkpoint is due, then nsp_diag_all,
// nsp_cross_sections_all and nsp_mean_profile_all, one batched call per kind for every
// member), so the driver is the same for both precisions and every member layout.
#include <dirent.h>
#include <sys/stat.h>
#include <sys/types.h>
#include <unistd.h>

#include <algorithm>
#include <array>
#include <cerrno>
#include <cinttypes>
#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include "nsp_internal.h"

namespace {

// Output files, in the reference's names (mod_io_nonlinear.cu:279, 296-297, 310).
enum { F_FRC, F_QCR, F_UCR, F_MNP, NFILES };
const char* const kFile[NFILES] = {"io_friction.txt", "io_qcross.txt", "io_ucross.txt", "io_meanpr.txt"};
// Accumulator (and interval) of each file: friction, cross sections (q and u), mean profile.
const int kClock[NFILES] = {0, 1, 1, 2};
const char* const kClockName[3] = {"acc_frc", "acc_qcr", "acc_mnp"};
// Restart files read by initField (mod_io_nonlinear.cu:426-429) and the final dump (main.cu:42-44).
const char* const kState[3] = {"ur_s.bin", "ut_s.bin", "uz_s.bin"};
const char* const kFinal[3] = {"ur.bin", "ut.bin", "uz.bin"};
const char* const kSidecar = "checkpoint.json";
const char* const kFormat = "nspipe-gb300 checkpoint";
constexpr int kVersion = 1;

std::string strf(const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  return buf;
}

std::string join(const std::string& a, const std::string& b) {
  if (a.empty() || b.empty()) return a.empty() ? b : a;
  return a.back() == '/' ? a + b : a + "/" + b;
}

bool is_dir(const std::string& p) {
  struct stat s;
  return stat(p.c_str(), &s) == 0 && S_ISDIR(s.st_mode);
}

bool is_file(const std::string& p) {
  struct stat s;
  return stat(p.c_str(), &s) == 0 && S_ISREG(s.st_mode);
}

long long file_size(const std::string& p) {
  struct stat s;
  return stat(p.c_str(), &s) == 0 && S_ISREG(s.st_mode) ? (long long)s.st_size : -1;
}

// mkdir -p
bool make_dirs(const std::string& p) {
  if (p.empty() || is_dir(p)) return true;
  size_t cut = p.find_last_of('/');
  if (cut != std::string::npos && cut > 0 && !make_dirs(p.substr(0, cut))) return false;
  return mkdir(p.c_str(), 0755) == 0 || errno == EEXIST;
}

// Removes a checkpoint directory: its files and its member_* subdirectories' files.
void remove_checkpoint_dir(const std::string& dir) {
  DIR* d = opendir(dir.c_str());
  if (!d) return;
  std::vector<std::string> names;
  while (dirent* e = readdir(d))
    if (strcmp(e->d_name, ".") && strcmp(e->d_name, "..")) names.push_back(e->d_name);
  closedir(d);
  for (const std::string& n : names) {
    std::string p = join(dir, n);
    if (is_dir(p) && n.compare(0, 7, "member_") == 0) {
      remove_checkpoint_dir(p);
    } else if (is_file(p)) {
      unlink(p.c_str());
    }
  }
  rmdir(dir.c_str());
}

// FNV-1a 64 of a file's bytes; false if unreadable.
bool fnv1a64(const std::string& path, uint64_t* out) {
  FILE* f = fopen(path.c_str(), "rb");
  if (!f) return false;
  uint64_t h = 14695981039346656037ull;
  std::vector<unsigned char> buf(1 << 20);
  size_t n;
  while ((n = fread(buf.data(), 1, buf.size(), f)) > 0)
    for (size_t i = 0; i < n; i++) h = (h ^ buf[i]) * 1099511628211ull;
  bool ok = !ferror(f);
  fclose(f);
  *out = h;
  return ok;
}

std::string e8(double v) { return strf("%.8e", v); }
std::string g17(double v) { return strf("%.17g", v); }

// ---- a small JSON reader for the sidecar -------------------------------------------
struct Json {
  enum Kind { NUL, BOOL, NUM, STR, ARR, OBJ } kind = NUL;
  double num = 0.0;
  std::string str;
  std::vector<Json> arr;
  std::vector<std::pair<std::string, Json>> obj;
  const Json* get(const char* key) const {
    for (const auto& kv : obj)
      if (kv.first == key) return &kv.second;
    return nullptr;
  }
};

struct JsonReader {
  const char* p;
  const char* end;
  bool ok = true;
  void ws() {
    while (p < end && (*p == ' ' || *p == '\n' || *p == '\r' || *p == '\t')) p++;
  }
  bool lit(const char* s) {
    size_t n = strlen(s);
    if ((size_t)(end - p) >= n && !strncmp(p, s, n)) {
      p += n;
      return true;
    }
    return false;
  }
  std::string string() {
    std::string s;
    if (p >= end || *p != '"') {
      ok = false;
      return s;
    }
    for (p++; p < end && *p != '"'; p++) {
      if (*p == '\\' && p + 1 < end) {
        p++;
        switch (*p) {
          case 'n': s += '\n'; break;
          case 't': s += '\t'; break;
          case 'r': s += '\r'; break;
          case 'b': s += '\b'; break;
          case 'f': s += '\f'; break;
          case 'u': {  // \u00XX only (the writer escapes control characters this way)
            if (end - p < 5) { ok = false; return s; }
            s += (char)strtol(std::string(p + 1, p + 5).c_str(), nullptr, 16);
            p += 4;
            break;
          }
          default: s += *p;
        }
      } else {
        s += *p;
      }
    }
    if (p >= end) ok = false;
    else p++;
    return s;
  }
  Json value(int depth = 0) {
    Json v;
    ws();
    if (p >= end || depth > 32) {
      ok = false;
      return v;
    }
    if (*p == '{') {
      v.kind = Json::OBJ;
      p++;
      ws();
      if (p < end && *p == '}') { p++; return v; }
      while (ok) {
        ws();
        std::string k = string();
        ws();
        if (p >= end || *p != ':') { ok = false; break; }
        p++;
        v.obj.emplace_back(k, value(depth + 1));
        ws();
        if (p < end && *p == ',') { p++; continue; }
        if (p < end && *p == '}') { p++; break; }
        ok = false;
      }
    } else if (*p == '[') {
      v.kind = Json::ARR;
      p++;
      ws();
      if (p < end && *p == ']') { p++; return v; }
      while (ok) {
        v.arr.push_back(value(depth + 1));
        ws();
        if (p < end && *p == ',') { p++; continue; }
        if (p < end && *p == ']') { p++; break; }
        ok = false;
      }
    } else if (*p == '"') {
      v.kind = Json::STR;
      v.str = string();
    } else if (lit("true")) {
      v.kind = Json::BOOL;
      v.num = 1;
    } else if (lit("false")) {
      v.kind = Json::BOOL;
    } else if (lit("null")) {
    } else {
      char* q = nullptr;
      std::string tok;
      while (p < end && strchr("+-0123456789.eE", *p)) tok += *p++;
      v.kind = Json::NUM;
      v.num = strtod(tok.c_str(), &q);
      if (tok.empty() || *q) ok = false;
    }
    return v;
  }
};

bool parse_json(const std::string& text, Json* out) {
  JsonReader r{text.data(), text.data() + text.size()};
  *out = r.value();
  r.ws();
  return r.ok && r.p == r.end;
}

std::string json_str(const std::string& s) {
  std::string o = "\"";
  for (char ch : s) {
    if (ch == '"' || ch == '\\') {
      o += '\\';
      o += ch;
    } else if ((unsigned char)ch < 0x20) {
      o += strf("\\u%04x", ch);
    } else {
      o += ch;
    }
  }
  return o + "\"";
}

bool read_text(const std::string& path, std::string* out) {
  FILE* f = fopen(path.c_str(), "rb");
  if (!f) return false;
  out->clear();
  char buf[65536];
  size_t n;
  while ((n = fread(buf, 1, sizeof buf, f)) > 0) out->append(buf, n);
  fclose(f);
  return true;
}

// ---- checkpoint lookup and validation (shared by resume and nsp_checkpoint_info) -----
std::string step_dir_name(long long step) { return strf("step_%010lld", step); }

// The checkpoint directory that `ckpt` names: itself if it holds a sidecar, else its
// step_* subdirectory with the highest step whose sidecar exists.
bool resolve_checkpoint(const std::string& ckpt, std::string* dir, std::string* why) {
  if (is_file(join(ckpt, kSidecar))) {
    *dir = ckpt;
    return true;
  }
  DIR* d = opendir(ckpt.c_str());
  if (!d) {
    *why = "checkpoint directory not found: " + ckpt;
    return false;
  }
  long long best = -1;
  while (dirent* e = readdir(d)) {
    long long s;
    char tail;
    if (sscanf(e->d_name, "step_%lld%c", &s, &tail) == 1 && s > best && is_file(join(join(ckpt, e->d_name), kSidecar)))
      best = s;
  }
  closedir(d);
  if (best < 0) {
    *why = "no complete checkpoint in " + ckpt;
    return false;
  }
  *dir = join(ckpt, step_dir_name(best));
  return true;
}

// Reads and checks a checkpoint: sidecar syntax, format, version, and every state file
// against its recorded size and checksum.
int load_checkpoint(const std::string& ckpt, std::string* dir, Json* side, std::string* text, std::string* why) {
  if (!resolve_checkpoint(ckpt, dir, why)) return NSP_ERR_IO;
  if (!read_text(join(*dir, kSidecar), text)) {
    *why = "cannot read " + join(*dir, kSidecar);
    return NSP_ERR_IO;
  }
  if (!parse_json(*text, side) || side->kind != Json::OBJ) {
    *why = "malformed " + join(*dir, kSidecar);
    return NSP_ERR_IO;
  }
  const Json* fmt = side->get("format");
  const Json* ver = side->get("version");
  const Json* mem = side->get("members");
  if (!fmt || fmt->str != kFormat || !ver || ver->num != kVersion || !mem || mem->kind != Json::ARR || mem->arr.empty()) {
    *why = "not a version-1 nspipe-gb300 checkpoint: " + join(*dir, kSidecar);
    return NSP_ERR_IO;
  }
  for (const Json& m : mem->arr) {
    const Json* sub = m.get("dir");
    const Json* st = m.get("state");
    if (!sub || !st || st->kind != Json::ARR || st->arr.size() != 3) {
      *why = "incomplete member record in " + join(*dir, kSidecar);
      return NSP_ERR_IO;
    }
    for (const Json& f : st->arr) {
      const Json* name = f.get("file");
      const Json* bytes = f.get("bytes");
      const Json* sum = f.get("fnv1a64");
      if (!name || !bytes || !sum) {
        *why = "incomplete state record in " + join(*dir, kSidecar);
        return NSP_ERR_IO;
      }
      std::string path = join(join(*dir, sub->str), name->str);
      long long sz = file_size(path);
      if (sz != (long long)bytes->num) {
        *why = strf("%s: %lld bytes, the checkpoint recorded %.0f", path.c_str(), sz, bytes->num);
        return NSP_ERR_IO;
      }
      uint64_t h = 0;
      if (!fnv1a64(path, &h) || strf("%016" PRIx64, h) != sum->str) {
        *why = path + ": checksum differs from the checkpoint's record";
        return NSP_ERR_IO;
      }
    }
  }
  return NSP_OK;
}

struct OutFile {
  std::string path;
  FILE* f = nullptr;
  std::string pending;  // formatted rows not yet written
  int rows = 0;
};

struct Member {
  nsp_params p{};
  std::string sub;  // output / checkpoint subdirectory: "" (one member) or member_NNNN
  int NZR = 0;
  double t = 0.0;
  long long step = 0;
  double acc[3] = {0.0, 0.0, 0.0};
  OutFile out[NFILES];
};

}  // namespace

struct nsp_run {
  nsp_ctx* ctx = nullptr;
  nsp_run_opts o{};
  std::string out_dir, ckpt_dir;
  int precision = NSP_FP64;
  long long step = 0;  // steps since t = 0 (all members advance together)
  std::vector<Member> mem;
  double interval[3] = {0.5, 0.5, 0.5};
};

namespace {

int fail(nsp_run* r, int code, const std::string& msg) { return nsp::ctx_fail(r ? r->ctx : nullptr, code, msg); }

bool files_on(const nsp_run* r, int f) { return !r->out_dir.empty() && r->interval[kClock[f]] >= 0.0; }

int write_pending(nsp_run* r, OutFile& of) {
  if (!of.f || of.pending.empty()) return NSP_OK;
  size_t put = fwrite(of.pending.data(), 1, of.pending.size(), of.f);
  if (put != of.pending.size() || fflush(of.f) != 0) return fail(r, NSP_ERR_IO, "writing error: " + of.path);
  of.pending.clear();
  of.rows = 0;
  return NSP_OK;
}

int flush_all(nsp_run* r) {
  for (Member& m : r->mem)
    for (OutFile& of : m.out)
      if (int rc = write_pending(r, of)) return rc;
  return NSP_OK;
}

int add_row(nsp_run* r, OutFile& of, const std::string& row) {
  of.pending += row;
  if (++of.rows >= std::max(1, r->o.rows_per_write)) return write_pending(r, of);
  return NSP_OK;
}

std::string value_row(double t, const double* v, int n) {
  std::string s = e8(t) + "  ";
  for (int i = 0; i < n; i++) s += e8(v[i]) + "  ";
  return s + "\n";
}

// Header rows of setIO (mod_io_nonlinear.cu:302-305, 314-315): 0 and the axial points
// z = LZ n / NZR of the cross-section files, 0 and the radial points of io_meanpr.txt.
std::string header_row(nsp_run* r, const Member& m, int f) {
  if (f == F_QCR || f == F_UCR) {
    std::vector<double> z(m.NZR);
    for (int i = 0; i < m.NZR; i++) z[i] = m.p.LZ * double(i) / double(m.NZR);
    return value_row(0.0, z.data(), m.NZR);
  }
  std::vector<double> rr(m.p.NR);
  nsp_grid(r->ctx, (int)(&m - r->mem.data()), rr.data(), nullptr);
  return value_row(0.0, rr.data(), m.p.NR);
}

// Opens the member's files: fresh (header row written) or, on resume, cut back to the
// size recorded at the checkpoint and appended to.
int open_files(nsp_run* r, Member& m, const Json* recorded) {
  if (r->out_dir.empty()) return NSP_OK;
  std::string dir = join(r->out_dir, m.sub);
  if (!make_dirs(dir)) return fail(r, NSP_ERR_IO, "cannot create " + dir);
  for (int f = 0; f < NFILES; f++) {
    if (!files_on(r, f)) continue;
    OutFile& of = m.out[f];
    of.path = join(dir, kFile[f]);
    const Json* size = recorded ? recorded->get(kFile[f]) : nullptr;
    if (size) {
      long long have = file_size(of.path), want = (long long)size->num;
      if (have < want)
        return fail(r, NSP_ERR_IO, strf("%s has %lld bytes, fewer than the %lld it had at the checkpoint",
                                        of.path.c_str(), have, want));
      if (truncate(of.path.c_str(), (off_t)want) != 0) return fail(r, NSP_ERR_IO, "cannot truncate " + of.path);
      of.f = fopen(of.path.c_str(), "ab");
      if (!of.f) return fail(r, NSP_ERR_IO, "cannot open " + of.path);
    } else {
      of.f = fopen(of.path.c_str(), "wb");
      if (!of.f) return fail(r, NSP_ERR_IO, "cannot open " + of.path);
      if (f != F_FRC) {  // io_friction.txt has no header row
        of.pending = header_row(r, m, f);
        if (int rc = write_pending(r, of)) return rc;
      }
    }
  }
  return NSP_OK;
}

int init_members(nsp_run* r) {
  int n = 0;
  if (int rc = nsp_info(r->ctx, &n, &r->precision)) return rc;
  r->mem.resize(n);
  for (int i = 0; i < n; i++) {
    Member& m = r->mem[i];
    if (int rc = nsp_get_params(r->ctx, i, &m.p)) return rc;
    m.sub = n > 1 ? strf("member_%04d", i) : "";
    m.NZR = 3 * (m.p.NZ - 1);
  }
  // the radial grid exists only after nsp_setup
  std::vector<double> probe(r->mem[0].p.NR);
  if (int rc = nsp_grid(r->ctx, 0, probe.data(), nullptr)) return rc;
  return NSP_OK;
}

nsp_run* new_run(nsp_ctx* ctx, const nsp_run_opts* o) {
  nsp_run* r = new nsp_run;
  r->ctx = ctx;
  r->o = *o;
  r->out_dir = o->out_dir ? o->out_dir : "";
  r->ckpt_dir = o->ckpt_dir ? o->ckpt_dir : "";
  r->o.out_dir = nullptr;  // the strings live in out_dir / ckpt_dir
  r->o.ckpt_dir = nullptr;
  r->interval[0] = o->dt_frc;
  r->interval[1] = o->dt_qcr;
  r->interval[2] = o->dt_mnp;
  return r;
}

int check_opts(nsp_ctx* ctx, const nsp_run_opts* o) {
  if (!ctx || !o) return NSP_ERR_ARG;
  if (o->rows_per_write < 1) return nsp::ctx_fail(ctx, NSP_ERR_ARG, "rows_per_write must be >= 1");
  if (o->ckpt_every < 0 || o->ckpt_keep < 0) return nsp::ctx_fail(ctx, NSP_ERR_ARG, "negative checkpoint schedule");
  if (o->ckpt_every > 0 && !o->ckpt_dir) return nsp::ctx_fail(ctx, NSP_ERR_ARG, "ckpt_every without ckpt_dir");
  if (std::isnan(o->dt_frc) || std::isnan(o->dt_qcr) || std::isnan(o->dt_mnp))
    return nsp::ctx_fail(ctx, NSP_ERR_ARG, "NaN output interval");
  return NSP_OK;
}

// Steps from accumulator acc until a row is due (at most cap).
int steps_until_due(double acc, double dt, double interval, int cap) {
  if (interval < 0.0) return cap;
  for (int j = 1; j <= cap; j++) {
    acc += dt;
    if (acc >= interval) return j;
  }
  return cap;
}

// Rows after a chunk whose last step made them due (due[member][kind]): wrt_frc,
// wrt_qcr + wrt_ucr, wrt_mpr in integrate's order (mod_integrate.cu:134-152).  Each
// kind is sampled for every member in one batched call when any member is due.
int sample(nsp_run* r, const std::vector<std::array<bool, 3>>& due, long long target) {
  const int n = (int)r->mem.size();
  bool any[3] = {false, false, false};
  for (int i = 0; i < n; i++)
    for (int c = 0; c < 3; c++) any[c] = any[c] || due[i][c];
  if (any[0]) {
    std::vector<nsp_diag_out> d(n);
    if (int rc = nsp_diag_all(r->ctx, d.data())) return rc;
    for (int i = 0; i < n; i++) {
      if (!due[i][0]) continue;
      Member& m = r->mem[i];
      if (r->o.verbose) {
        printf("\n err=%e\n", d[i].last_err);
        if (n > 1) printf(" Step %lld of %lld (member %d)\n", m.step, target, i);
        else printf(" Step %lld of %lld\n", m.step, target);
      }
      if (m.out[F_FRC].f)
        if (int rc = add_row(r, m.out[F_FRC], e8(m.t) + "  " + e8(d[i].u_centre) + "  " + e8(d[i].u_tau) + "\n"))
          return rc;
    }
  }
  if (any[1]) {
    size_t tot = 0;
    for (const Member& m : r->mem) tot += m.NZR;
    std::vector<double> q(tot), u(tot);
    if (int rc = nsp_cross_sections_all(r->ctx, q.data(), u.data())) return rc;
    size_t o = 0;
    for (int i = 0; i < n; i++) {
      Member& m = r->mem[i];
      if (due[i][1]) {
        if (m.out[F_QCR].f)
          if (int rc = add_row(r, m.out[F_QCR], value_row(m.t, q.data() + o, m.NZR))) return rc;
        if (m.out[F_UCR].f)
          if (int rc = add_row(r, m.out[F_UCR], value_row(m.t, u.data() + o, m.NZR))) return rc;
      }
      o += m.NZR;
    }
  }
  if (any[2]) {
    size_t tot = 0;
    for (const Member& m : r->mem) tot += m.p.NR;
    std::vector<double> prof(tot);
    if (int rc = nsp_mean_profile_all(r->ctx, prof.data())) return rc;
    size_t o = 0;
    for (int i = 0; i < n; i++) {
      Member& m = r->mem[i];
      if (due[i][2] && m.out[F_MNP].f)
        if (int rc = add_row(r, m.out[F_MNP], value_row(m.t, prof.data() + o, m.p.NR))) return rc;
      o += m.p.NR;
    }
  }
  return NSP_OK;
}

std::string precision_name(int p) { return p == NSP_MIXED ? "mixed" : "fp64"; }

int write_checkpoint(nsp_run* r) {
  if (r->ckpt_dir.empty()) return fail(r, NSP_ERR_STATE, "the run has no checkpoint directory");
  if (int rc = flush_all(r)) return rc;
  const std::string dir = join(r->ckpt_dir, step_dir_name(r->step));
  if (is_dir(dir)) remove_checkpoint_dir(dir);
  if (!make_dirs(dir)) return fail(r, NSP_ERR_IO, "cannot create " + dir);
  std::string js = "{\n  \"format\": " + json_str(kFormat) + ",\n  \"version\": " + strf("%d", kVersion) +
                   ",\n  \"precision\": " + json_str(precision_name(r->precision)) + ",\n  \"step\": " +
                   strf("%lld", r->step) + ",\n  \"out_dir\": " + json_str(r->out_dir) + ",\n  \"members\": [";
  for (size_t i = 0; i < r->mem.size(); i++) {
    Member& m = r->mem[i];
    const std::string mdir = join(dir, m.sub);
    if (!make_dirs(mdir)) return fail(r, NSP_ERR_IO, "cannot create " + mdir);
    std::string f[3];
    for (int c = 0; c < 3; c++) f[c] = join(mdir, kState[c]);
    if (int rc = nsp_save_state(r->ctx, (int)i, f[0].c_str(), f[1].c_str(), f[2].c_str())) return rc;
    const nsp_params& p = m.p;
    js += std::string(i ? "," : "") + "\n    {\"dir\": " + json_str(m.sub.empty() ? "." : m.sub);
    js += strf(", \"NR\": %d, \"NT\": %d, \"NZ\": %d, \"maxit\": %d, \"sten\": %d", p.NR, p.NT, p.NZ, p.maxit, p.sten);
    const std::pair<const char*, double> dv[] = {{"LT", p.LT}, {"LZ", p.LZ}, {"Re", p.Re}, {"dt", p.dt}, {"d_im", p.d_im},
                                                 {"tol", p.tol}, {"Qdes", p.Qdes}, {"t", m.t}, {"acc_frc", m.acc[0]},
                                                 {"acc_qcr", m.acc[1]}, {"acc_mnp", m.acc[2]}};
    for (const auto& kv : dv) js += strf(", \"%s\": ", kv.first) + g17(kv.second);
    js += strf(", \"step\": %lld,\n     \"state\": [", m.step);
    for (int c = 0; c < 3; c++) {
      uint64_t h = 0;
      if (!fnv1a64(f[c], &h)) return fail(r, NSP_ERR_IO, "cannot read back " + f[c]);
      js += strf("%s{\"file\": \"%s\", \"bytes\": %lld, \"fnv1a64\": \"%016" PRIx64 "\"}", c ? ", " : "", kState[c],
                 file_size(f[c]), h);
    }
    js += "],\n     \"outputs\": {";
    bool first = true;
    for (int k = 0; k < NFILES; k++) {
      if (!m.out[k].f) continue;
      js += strf("%s\"%s\": %lld", first ? "" : ", ", kFile[k], file_size(m.out[k].path));
      first = false;
    }
    js += "}}";
  }
  js += "\n  ]\n}\n";
  // The sidecar goes last, under a temporary name renamed into place: a directory
  // without checkpoint.json is an incomplete checkpoint and is never resumed from.
  const std::string tmp = join(dir, std::string(kSidecar) + ".tmp");
  FILE* fh = fopen(tmp.c_str(), "wb");
  if (!fh) return fail(r, NSP_ERR_IO, "cannot write " + tmp);
  bool ok = fwrite(js.data(), 1, js.size(), fh) == js.size();
  ok = (fflush(fh) == 0) && ok;
  ok = (fsync(fileno(fh)) == 0) && ok;
  ok = (fclose(fh) == 0) && ok;
  if (!ok || rename(tmp.c_str(), join(dir, kSidecar).c_str()) != 0)
    return fail(r, NSP_ERR_IO, "cannot write " + join(dir, kSidecar));
  // Checkpoints past this step belong to a timeline that was abandoned when the run
  // resumed from an older one: remove them.  Then keep the newest ckpt_keep complete
  // checkpoints and drop incomplete ones older than this.
  {
    std::vector<std::pair<long long, bool>> found;
    if (DIR* d = opendir(r->ckpt_dir.c_str())) {
      while (dirent* e = readdir(d)) {
        long long s;
        char tail;
        if (sscanf(e->d_name, "step_%lld%c", &s, &tail) == 1 && strlen(e->d_name) == 15)
          found.emplace_back(s, is_file(join(join(r->ckpt_dir, e->d_name), kSidecar)));
      }
      closedir(d);
    }
    std::sort(found.begin(), found.end(), [](const auto& a, const auto& b) { return a.first > b.first; });
    int kept = 0;
    for (const auto& fs : found) {
      if (fs.first > r->step) {
        remove_checkpoint_dir(join(r->ckpt_dir, step_dir_name(fs.first)));
        continue;
      }
      if (fs.second && (r->o.ckpt_keep == 0 || kept < r->o.ckpt_keep)) {
        kept++;
        continue;
      }
      remove_checkpoint_dir(join(r->ckpt_dir, step_dir_name(fs.first)));
    }
  }
  return NSP_OK;
}

bool same_params(const nsp_params& a, const Json& m, std::string* which) {
  const std::pair<const char*, double> v[] = {{"NR", a.NR}, {"NT", a.NT}, {"NZ", a.NZ}, {"LT", a.LT}, {"LZ", a.LZ},
                                              {"Re", a.Re}, {"dt", a.dt}, {"d_im", a.d_im}, {"maxit", a.maxit},
                                              {"tol", a.tol}, {"sten", a.sten}, {"Qdes", a.Qdes}};
  for (const auto& kv : v) {
    const Json* j = m.get(kv.first);
    if (!j || j->kind != Json::NUM || j->num != kv.second) {
      *which = strf("%s: checkpoint %s, context %.17g", kv.first, j ? g17(j->num).c_str() : "missing", kv.second);
      return false;
    }
  }
  return true;
}

void close_files(nsp_run* r) {
  for (Member& m : r->mem)
    for (OutFile& of : m.out)
      if (of.f) {
        fclose(of.f);
        of.f = nullptr;
      }
}

}  // namespace

extern "C" {

int nsp_run_default_opts(nsp_run_opts* o) {
  if (!o) return NSP_ERR_ARG;
  o->out_dir = ".";
  o->dt_frc = 0.5;  // head.h:33-40
  o->dt_qcr = 0.5;
  o->dt_mnp = 0.5;
  o->rows_per_write = 100;
  o->ckpt_dir = nullptr;
  o->ckpt_every = 0;
  o->ckpt_keep = 2;
  o->final_state = 1;
  o->verbose = 0;
  return NSP_OK;
}

int nsp_output_schedule(double dt, double interval, int nsteps, double* acc, unsigned char* due) {
  if (!acc || nsteps < 0 || (nsteps > 0 && !due)) return NSP_ERR_ARG;
  for (int j = 0; j < nsteps; j++) {
    *acc += dt;  // t_frc += dt (mod_integrate.cu:131)
    due[j] = interval >= 0.0 && *acc >= interval;
    if (due[j]) *acc = 0.0;  // t_frc = 0.0 (:138)
  }
  return NSP_OK;
}

int nsp_run_open(nsp_ctx* ctx, const nsp_run_opts* o, nsp_run** out) {
  if (!out) return NSP_ERR_ARG;
  *out = nullptr;
  if (int rc = check_opts(ctx, o)) return rc;
  nsp_run* r = new_run(ctx, o);
  int rc = init_members(r);
  for (size_t i = 0; rc == NSP_OK && i < r->mem.size(); i++) rc = open_files(r, r->mem[i], nullptr);
  if (rc == NSP_OK && !r->ckpt_dir.empty() && !make_dirs(r->ckpt_dir)) rc = fail(r, NSP_ERR_IO, "cannot create " + r->ckpt_dir);
  if (rc != NSP_OK) {
    close_files(r);
    delete r;
    return rc;
  }
  *out = r;
  return NSP_OK;
}

int nsp_run_resume(nsp_ctx* ctx, const nsp_run_opts* o, const char* ckpt, nsp_run** out) {
  if (!out) return NSP_ERR_ARG;
  *out = nullptr;
  if (int rc = check_opts(ctx, o)) return rc;
  if (!ckpt) return nsp::ctx_fail(ctx, NSP_ERR_ARG, "null checkpoint path");
  std::string dir, text, why;
  Json side;
  if (int rc = load_checkpoint(ckpt, &dir, &side, &text, &why)) return nsp::ctx_fail(ctx, rc, why);
  nsp_run* r = new_run(ctx, o);
  auto bail = [&](int rc) {
    close_files(r);
    delete r;
    return rc;
  };
  if (int rc = init_members(r)) return bail(rc);
  const Json& mem = *side.get("members");
  if (mem.arr.size() != r->mem.size())
    return bail(fail(r, NSP_ERR_ARG, strf("the checkpoint holds %zu members, the context %zu", mem.arr.size(), r->mem.size())));
  const Json* step = side.get("step");
  if (!step || step->kind != Json::NUM) return bail(fail(r, NSP_ERR_IO, "checkpoint without a step count"));
  r->step = (long long)step->num;
  for (size_t i = 0; i < r->mem.size(); i++) {
    Member& m = r->mem[i];
    const Json& rec = mem.arr[i];
    if (!same_params(m.p, rec, &why)) return bail(fail(r, NSP_ERR_ARG, strf("member %zu: ", i) + why));
    const Json* t = rec.get("t");
    const Json* ms = rec.get("step");
    if (!t || !ms) return bail(fail(r, NSP_ERR_IO, "checkpoint member without time"));
    m.t = t->num;
    m.step = (long long)ms->num;
    for (int k = 0; k < 3; k++) {
      const Json* a = rec.get(kClockName[k]);
      if (!a) return bail(fail(r, NSP_ERR_IO, "checkpoint member without output accumulators"));
      m.acc[k] = a->num;
    }
    const std::string mdir = join(dir, rec.get("dir")->str);
    std::string f[3];
    for (int c = 0; c < 3; c++) f[c] = join(mdir, kState[c]);
    if (int rc = nsp_load_state(ctx, (int)i, f[0].c_str(), f[1].c_str(), f[2].c_str())) return bail(rc);
    if (int rc = open_files(r, m, rec.get("outputs"))) return bail(rc);
  }
  if (!r->ckpt_dir.empty() && !make_dirs(r->ckpt_dir)) return bail(fail(r, NSP_ERR_IO, "cannot create " + r->ckpt_dir));
  *out = r;
  return NSP_OK;
}

int nsp_run_advance(nsp_run* r, int nsteps, int* iters_out) {
  if (!r || nsteps < 0) return NSP_ERR_ARG;
  const int n = (int)r->mem.size();
  const long long target = r->step + nsteps;
  std::vector<int> it;
  int done = 0;
  while (done < nsteps) {
    int k = nsteps - done;
    for (const Member& m : r->mem)
      for (int c = 0; c < 3; c++) {
        bool on = false;
        for (int f = 0; f < NFILES; f++) on = on || (kClock[f] == c && m.out[f].f);
        if (on || (c == 0 && r->o.verbose)) k = steps_until_due(m.acc[c], m.p.dt, r->interval[c], k);
      }
    if (r->o.ckpt_every > 0) k = (int)std::min<long long>(k, r->o.ckpt_every - r->step % r->o.ckpt_every);
    it.assign((size_t)k * n, 0);
    int rc = nsp_step(r->ctx, k, it.data());
    if (rc != NSP_OK && rc != NSP_ERR_NONFINITE && rc != NSP_ERR_MAXIT) return rc;
    if (iters_out) std::copy(it.begin(), it.end(), iters_out + (size_t)done * n);
    r->step += k;
    done += k;
    std::vector<std::array<bool, 3>> due(n);
    for (int i = 0; i < n; i++) {
      Member& m = r->mem[i];
      due[i] = {false, false, false};
      for (int j = 0; j < k; j++) {  // c_t++; t += dt; t_frc += dt; ... (mod_integrate.cu:131)
        m.step++;
        m.t += m.p.dt;
        for (int c = 0; c < 3; c++) {
          m.acc[c] += m.p.dt;
          due[i][c] = r->interval[c] >= 0.0 && m.acc[c] >= r->interval[c];
          if (due[i][c]) m.acc[c] = 0.0;
        }
      }
      // a row only where the member writes that file, or prints progress
      due[i][0] = due[i][0] && (m.out[F_FRC].f || r->o.verbose);
      due[i][1] = due[i][1] && (m.out[F_QCR].f || m.out[F_UCR].f);
      due[i][2] = due[i][2] && m.out[F_MNP].f;
    }
    if (int s = sample(r, due, target)) return s;
    if (rc == NSP_ERR_NONFINITE || rc == NSP_ERR_MAXIT) {  // rows of the chunk, no checkpoint
      flush_all(r);
      return rc;
    }
    if (r->o.ckpt_every > 0 && r->step % r->o.ckpt_every == 0)
      if (int c = write_checkpoint(r)) return c;
  }
  return NSP_OK;
}

int nsp_run_checkpoint(nsp_run* r) {
  if (!r) return NSP_ERR_ARG;
  return write_checkpoint(r);
}

int nsp_run_time(nsp_run* r, int member, double* t, long long* steps) {
  if (!r) return NSP_ERR_ARG;
  if (member < 0 || member >= (int)r->mem.size()) return fail(r, NSP_ERR_ARG, strf("member %d out of range", member));
  if (t) *t = r->mem[member].t;
  if (steps) *steps = r->mem[member].step;
  return NSP_OK;
}

int nsp_run_close(nsp_run* r) {
  if (!r) return NSP_OK;
  int rc = flush_all(r);
  if (rc == NSP_OK && r->o.final_state && !r->out_dir.empty()) {
    for (size_t i = 0; rc == NSP_OK && i < r->mem.size(); i++) {
      std::string dir = join(r->out_dir, r->mem[i].sub);
      if (!make_dirs(dir)) {
        rc = fail(r, NSP_ERR_IO, "cannot create " + dir);
        break;
      }
      std::string f[3];
      for (int c = 0; c < 3; c++) f[c] = join(dir, kFinal[c]);
      rc = nsp_save_state(r->ctx, (int)i, f[0].c_str(), f[1].c_str(), f[2].c_str());
    }
  }
  close_files(r);
  delete r;
  return rc;
}

int nsp_checkpoint_info(const char* ckpt, char* json, int json_cap, char* path, int path_cap) {
  if (!ckpt) return NSP_ERR_ARG;
  std::string dir, text, why;
  Json side;
  if (int rc = load_checkpoint(ckpt, &dir, &side, &text, &why)) return nsp::ctx_fail(nullptr, rc, why);
  if (json) {
    if ((int)text.size() + 1 > json_cap) return NSP_ERR_ARG;
    memcpy(json, text.c_str(), text.size() + 1);
  }
  if (path) {
    if ((int)dir.size() + 1 > path_cap) return NSP_ERR_ARG;
    memcpy(path, dir.c_str(), dir.size() + 1);
  }
  return NSP_OK;
}

}  // extern "C"
