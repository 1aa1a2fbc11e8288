// sisi4s-gb300: the YAML step runner of the GB300 CCSD(T) library.
//
// Mirrors the host contract of sisi4s for its closed-shell CCSD(T) path:
// - the input file is a list of steps {name, in: {...}, out: {...}, note,
//   fallible, disable/enable} (src/Parser.cxx:21-72); "$Name" values are data
//   symbols, other values become anonymous Integer/Real/Text constants tried
//   in that order (src/Parser.cxx:35-58);
// - algorithms are created by name from a registry (src/algorithms/Algorithm.hpp:104-183)
//   and read/write named arguments with the same keys and defaults;
// - a step marked fallible catches its error and the run continues
//   (src/Sisi4s.cxx:71-84);
// - command line -i/--in, -o/--out, -l/--log, --dry, --log-level, --list
//   (src/Options.cxx:9-39).
// The arithmetic runs on the GPU through the C ABI in include/gbcc.h.
#include <gbcc.h>

#include <algorithm>
#include <chrono>
#include <cctype>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <functional>
#include <iomanip>
#include <iostream>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "yaml_lite.hpp"

namespace {

// ------------------------------------------------------------------ output
// Minimal ordered JSON value; JSON is valid YAML 1.2, so the output file can
// be read like the reference's sisi4s.out.yaml.
struct Json {
  enum K { Null, Num, Str, Arr, Obj } k = Null;
  double num = 0;
  std::string s;
  std::vector<Json> arr;
  std::vector<std::pair<std::string, Json>> obj;
  Json() = default;
  Json(double v) : k(Num), num(v) {}
  Json(int v) : k(Num), num(v) {}
  Json(long long v) : k(Num), num((double)v) {}
  Json(const std::string &v) : k(Str), s(v) {}
  Json(const char *v) : k(Str), s(v) {}
  static Json object() { Json j; j.k = Obj; return j; }
  static Json array() { Json j; j.k = Arr; return j; }
  Json &operator[](const std::string &key) {
    if (k != Obj) { k = Obj; obj.clear(); }
    for (auto &kv : obj)
      if (kv.first == key) return kv.second;
    obj.emplace_back(key, Json());
    return obj.back().second;
  }
  void push(const Json &v) { k = Arr; arr.push_back(v); }
  void dump(std::ostream &o, int ind = 0) const {
    const std::string pad(ind, ' ');
    switch (k) {
      case Null: o << "null"; break;
      case Num: {
        if (std::isfinite(num)) {
          char b[64];
          std::snprintf(b, sizeof b, "%.17g", num);
          o << b;
        } else {
          o << "null";
        }
        break;
      }
      case Str: {
        o << '"';
        for (char c : s) {
          if (c == '"' || c == '\\') o << '\\' << c;
          else if (c == '\n') o << "\\n";
          else o << c;
        }
        o << '"';
        break;
      }
      case Arr: {
        o << "[";
        for (size_t i = 0; i < arr.size(); ++i) {
          o << (i ? ",\n" : "\n") << pad << "  ";
          arr[i].dump(o, ind + 2);
        }
        o << (arr.empty() ? "]" : "\n" + pad + "]");
        break;
      }
      case Obj: {
        o << "{";
        for (size_t i = 0; i < obj.size(); ++i) {
          o << (i ? ",\n" : "\n") << pad << "  \"" << obj[i].first << "\": ";
          obj[i].second.dump(o, ind + 2);
        }
        o << (obj.empty() ? "}" : "\n" + pad + "}");
        break;
      }
    }
  }
};

int g_log_level = 1;
std::ofstream g_log;

void log(int level, const std::string &tag, const std::string &msg) {
  if (level > g_log_level) return;
  std::cout << tag << ": " << msg << std::endl;
  if (g_log) g_log << tag << ": " << msg << std::endl;
}

// -------------------------------------------------------------------- data
struct HTensor {
  std::vector<int64_t> lens;
  std::vector<double> re, im;  // column-major (first index fastest)
  bool complex = false;
  int64_t size() const {
    int64_t s = 1;
    for (auto l : lens) s *= l;
    return s;
  }
};

struct Data {
  enum Kind { Unset, Tensor, Real, Integer, Text } kind = Unset;
  std::string name;
  double real = 0;
  long long integer = 0;
  std::string text;
  std::shared_ptr<HTensor> tensor;
};

std::map<std::string, std::shared_ptr<Data>> g_data;
int g_anon = 0;

std::shared_ptr<Data> data_symbol(const std::string &name) {
  auto &d = g_data[name];
  if (!d) {
    d = std::make_shared<Data>();
    d->name = name;
  }
  return d;
}

std::shared_ptr<Data> anon(Data::Kind k) {
  static const char *names[] = {"Unset", "Tensor", "Real", "Integer", "Text"};
  auto d = std::make_shared<Data>();
  d->kind = k;
  d->name = std::string(names[k]) + std::to_string(g_anon++);
  g_data[d->name] = d;
  return d;
}

struct StepError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

// ------------------------------------------------------------ GPU context
gbcc_ctx *g_ctx = nullptr;

gbcc_ctx *gpu() {
  if (!g_ctx) {
    gbcc_status st = gbcc_ctx_create(0, nullptr, &g_ctx);
    if (st != GBCC_OK)
      throw StepError(std::string("GPU context: ") + gbcc_status_string(st) +
                      ": " + gbcc_last_error(nullptr));
  }
  return g_ctx;
}

void check(gbcc_status st, const char *what, bool allow_not_converged = false) {
  if (st == GBCC_OK) return;
  if (allow_not_converged && st == GBCC_NOT_CONVERGED) return;
  throw StepError(std::string(what) + ": " + gbcc_status_string(st) + ": " +
                  gbcc_last_error(g_ctx));
}

// --------------------------------------------------------------- algorithm
struct Algorithm {
  std::string name, note;
  bool fallible = false;
  std::vector<std::pair<std::string, std::string>> args;  // key -> data name
  Json emit = Json::object();
  virtual ~Algorithm() = default;
  virtual void run() = 0;

  bool given(const std::string &k) const {
    for (auto &a : args)
      if (a.first == k) return true;
    return false;
  }
  std::shared_ptr<Data> arg(const std::string &k) const {
    for (auto &a : args)
      if (a.first == k) return data_symbol(a.second);
    throw StepError("argument " + k + " missing in " + name);
  }
  std::string text(const std::string &k) const {
    auto d = arg(k);
    if (d->kind != Data::Text) throw StepError("argument " + k + " is not text");
    return d->text;
  }
  std::string text(const std::string &k, const std::string &def) const {
    return given(k) ? text(k) : def;
  }
  long long integer(const std::string &k, long long def) const {
    if (!given(k)) return def;
    auto d = arg(k);
    if (d->kind == Data::Integer) return d->integer;
    throw StepError("argument " + k + " is not an integer");
  }
  // Real arguments accept integers and real data (Algorithm.cxx:100-133)
  double real(const std::string &k) const {
    auto d = arg(k);
    if (d->kind == Data::Real) return d->real;
    if (d->kind == Data::Integer) return (double)d->integer;
    if (d->kind == Data::Tensor && d->tensor->size() == 1) return d->tensor->re[0];
    throw StepError("argument " + k + " is not real");
  }
  double real(const std::string &k, double def) const {
    return given(k) ? real(k) : def;
  }
  HTensor &tensor(const std::string &k) const {
    auto d = arg(k);
    if (d->kind == Data::Real) {
      auto t = std::make_shared<HTensor>();
      t->re = {d->real};
      d->tensor = t;
      return *t;
    }
    if (d->kind != Data::Tensor || !d->tensor)
      throw StepError("argument " + k + " (" + d->name + ") is not a tensor");
    return *d->tensor;
  }
  // The ABI takes bare pointers, so every tensor handed to it must have
  // exactly the lengths of the reference's tensor for that key.
  const HTensor &tensor(const std::string &k, const std::vector<int64_t> &lens) const {
    const HTensor &t = tensor(k);
    if (t.lens != lens) throw StepError("argument " + k + " has lengths " + lens_str(t.lens) +
                                        ", expected " + lens_str(lens));
    return t;
  }
  const double *tensor_or_null(const std::string &k, const std::vector<int64_t> &lens) const {
    return given(k) ? tensor(k, lens).re.data() : nullptr;
  }
  static std::string lens_str(const std::vector<int64_t> &l) {
    std::string s = "[";
    for (size_t i = 0; i < l.size(); ++i) s += (i ? "," : "") + std::to_string(l[i]);
    return s + "]";
  }
  void set_tensor(const std::string &k, std::shared_ptr<HTensor> t) {
    auto d = arg(k);
    d->kind = Data::Tensor;
    d->tensor = std::move(t);
  }
  void set_real(const std::string &k, double v) {
    auto d = arg(k);
    d->kind = Data::Real;
    d->real = v;
  }
};

using Factory = std::function<std::unique_ptr<Algorithm>()>;
std::map<std::string, Factory> &registry() {
  static std::map<std::string, Factory> r;
  return r;
}
struct Registrar {
  Registrar(const std::string &n, Factory f) { registry()[n] = std::move(f); }
};
#define REGISTER_ALGORITHM(NAME) \
  static Registrar reg_##NAME(#NAME, [] { return std::unique_ptr<Algorithm>(new NAME()); })

// ----------------------------------------------------------- tensor files
// cc4s format: YAML header (version, type, dimensions, scalarType,
// elements.type, unit) plus a .elements file, text (one value per line) or
// IEEE binary, first index fastest (src/algorithms/Read.cxx:25-98).
std::string replace_ext(const std::string &p, const std::string &ext) {
  const size_t slash = p.find_last_of('/');
  const size_t dot = p.find_last_of('.');
  if (dot == std::string::npos || (slash != std::string::npos && dot < slash))
    return p + "." + ext;
  return p.substr(0, dot) + "." + ext;
}

std::shared_ptr<HTensor> read_cc4s(const std::string &file) {
  auto h = yl::parse_file(file);
  if (!h->is_map()) throw StepError(file + ": header is not a map");
  for (const char *k : {"dimensions", "elements", "scalarType", "type", "unit", "version"})
    if (!h->get(k)) throw StepError(file + ": header key " + k + " missing");
  auto t = std::make_shared<HTensor>();
  auto dims = h->get("dimensions");
  if (!dims->is_seq() && dims->kind != yl::Node::Null)
    throw StepError(file + ": dimensions must be a list");
  int64_t n = 1;
  for (auto &d : dims->seq) {
    auto len = d->is_map() ? d->get("length") : nullptr;
    if (!len) throw StepError(file + ": a dimension has no length");
    const long long l = len->as_int();
    // the element count must fit a signed 64-bit byte count of Complex64 data
    if (l < 0 || (l > 0 && n > (INT64_MAX / 16) / l))
      throw StepError(file + ": bad dimension length " + std::to_string(l));
    n *= l;
    t->lens.push_back(l);
  }
  auto elements = h->get("elements");
  auto etype = elements->is_map() ? elements->get("type") : nullptr;
  if (!etype) throw StepError(file + ": elements.type missing");
  const std::string st = h->get("scalarType")->str();
  const std::string et = etype->str();
  const std::string ef = replace_ext(file, "elements");
  if (st == "Real64") {
    t->re.resize(n);
    if (et == "TextFile") {
      std::ifstream f(ef);
      if (!f) throw StepError("cannot open " + ef);
      std::string line;
      int64_t i = 0;
      while (i < n && std::getline(f, line)) t->re[i++] = std::atof(line.c_str());
      if (i != n) throw StepError(ef + ": too few elements");
    } else if (et == "IeeeBinaryFile") {
      std::ifstream f(ef, std::ios::binary);
      if (!f.read(reinterpret_cast<char *>(t->re.data()), 8 * n))
        throw StepError(ef + ": too few elements");
    } else {
      throw StepError(file + ": unknown elements type " + et);
    }
  } else if (st == "Complex64") {
    t->complex = true;
    std::vector<double> buf(2 * n);
    std::ifstream f(ef, std::ios::binary);
    if (!f.read(reinterpret_cast<char *>(buf.data()), 16 * n))
      throw StepError(ef + ": too few elements");
    t->re.resize(n);
    t->im.resize(n);
    for (int64_t i = 0; i < n; ++i) {
      t->re[i] = buf[2 * i];
      t->im[i] = buf[2 * i + 1];
    }
  } else {
    throw StepError(file + ": unknown scalarType " + st);
  }
  return t;
}

void write_cc4s(const std::string &file, const HTensor &t, bool binary) {
  const std::string ef = replace_ext(file, "elements");
  const std::string hf = replace_ext(file, "yaml");
  {
    std::ofstream h(hf);
    h << "version: 100\ntype: Tensor\ndimensions:\n";
    for (auto l : t.lens) h << "  - length: " << l << "\n    type: State\n";
    h << "scalarType: " << (t.complex ? "Complex64" : "Real64") << "\n";
    h << "elements:\n  type: " << (binary ? "IeeeBinaryFile" : "TextFile") << "\n";
    h << "unit: 1\n";
  }
  if (binary) {
    std::ofstream f(ef, std::ios::binary);
    if (t.complex) {
      for (int64_t i = 0; i < t.size(); ++i) {
        f.write(reinterpret_cast<const char *>(&t.re[i]), 8);
        f.write(reinterpret_cast<const char *>(&t.im[i]), 8);
      }
    } else {
      f.write(reinterpret_cast<const char *>(t.re.data()), 8 * t.size());
    }
  } else {
    std::ofstream f(ef);
    f << std::setprecision(17);
    for (int64_t i = 0; i < t.size(); ++i) f << t.re[i] << "\n";
  }
}

// ------------------------------------------------------------- algorithms
struct Nop : Algorithm {
  void run() override {}
};
REGISTER_ALGORITHM(Nop);

struct Read : Algorithm {
  void run() override {
    auto t = read_cc4s(text("fileName"));
    emit["dimensions"] = (long long)t->lens.size();
    set_tensor("destination", t);
  }
};
REGISTER_ALGORITHM(Read);

struct Write : Algorithm {
  void run() override {
    auto d = arg("source");
    const bool binary = integer("binary", 1) != 0;
    write_cc4s(text("fileName", d->name), tensor("source"), binary);
  }
};
REGISTER_ALGORITHM(Write);

// ------------------------------------------------ TensorWriter / Reader
// The formats of src/util/TensorIo.cxx and src/util/BinaryTensorFormat.hpp.
//
// Text (:158-226): a line "name<d>order<d>len0<d>len1...", a line
// "rowIndexOrder<d>columnIndexOrder", then one line per row with the column
// elements separated by the delimiter; index letters are 'i' + dim; without
// orders every element is one row, first index fastest.  Numbers are written
// with 16 significant digits, complex ones as "(re,im)".
//
// Binary (:120-155): a 32-byte header {"TENS", int32 version 0x9000, "IEEE",
// int32 bytes per number, int32 numbers per element, int32 order, int32 flags,
// int32 reserved}, one 8-byte header {int32 length, char index name 'a'+dim,
// int8 flags, int16 reserved} per dimension, then the dense data (first index
// fastest, complex as (re, im) pairs).

// element offsets of the layout a text file is written in: dims of
// columnIndexOrder (fastest first), then those of rowIndexOrder
std::vector<int64_t> text_layout(const HTensor &t, const std::string &rows,
                                 const std::string &cols, int64_t *ncols) {
  const int order = (int)t.lens.size();
  const std::string all = cols + rows;
  std::vector<int> used(order, 0);
  if ((int)all.size() != order)
    throw StepError("rowIndexOrder and columnIndexOrder must hold the tensor's " +
                    std::to_string(order) + " indices");
  std::vector<int> dims;
  for (char c : all) {
    const int d = c - 'i';
    if (d < 0 || d >= order || used[d]++)
      throw StepError(std::string("bad index '") + c + "' in the index orders");
    dims.push_back(d);
  }
  std::vector<int64_t> stride(order, 1);
  for (int d = 1; d < order; ++d) stride[d] = stride[d - 1] * t.lens[d - 1];
  *ncols = 1;
  for (size_t q = 0; q < cols.size(); ++q) *ncols *= t.lens[dims[q]];
  std::vector<int64_t> off((size_t)t.size());
  std::vector<int64_t> idx(order, 0);
  for (int64_t e = 0; e < t.size(); ++e) {
    int64_t o = 0;
    for (int q = 0; q < order; ++q) o += idx[q] * stride[dims[q]];
    off[e] = o;
    for (int q = 0; q < order; ++q) {
      if (++idx[q] < t.lens[dims[q]]) break;
      idx[q] = 0;
    }
  }
  return off;
}

const char kMagic[4] = {'T', 'E', 'N', 'S'};
const char kIeee[4] = {'I', 'E', 'E', 'E'};
const int32_t kBinaryVersion = 0x09000;

template <class T>
void put(std::ostream &f, T v) {
  f.write(reinterpret_cast<const char *>(&v), sizeof v);
}
template <class T>
T get(std::istream &f, const std::string &file) {
  T v;
  if (!f.read(reinterpret_cast<char *>(&v), sizeof v)) throw StepError(file + ": truncated");
  return v;
}

void write_tensor_binary(const std::string &file, const HTensor &t) {
  std::ofstream f(file, std::ios::binary);
  if (!f) throw StepError("cannot open " + file);
  f.write(kMagic, 4);
  put<int32_t>(f, kBinaryVersion);
  f.write(kIeee, 4);
  put<int32_t>(f, t.complex ? 16 : 8);
  put<int32_t>(f, t.complex ? 2 : 1);
  put<int32_t>(f, (int32_t)t.lens.size());
  put<int32_t>(f, 0);
  put<int32_t>(f, 0);
  for (size_t d = 0; d < t.lens.size(); ++d) {
    put<int32_t>(f, (int32_t)t.lens[d]);
    put<char>(f, (char)('a' + d));
    put<int8_t>(f, 0);
    put<int16_t>(f, 0);
  }
  for (int64_t e = 0; e < t.size(); ++e) {
    put<double>(f, t.re[e]);
    if (t.complex) put<double>(f, t.im[e]);
  }
}

std::shared_ptr<HTensor> read_tensor_binary(const std::string &file, bool complex) {
  std::ifstream f(file, std::ios::binary);
  if (!f) throw StepError("Failed to open file \"" + file + "\"");
  char magic[4], type[4];
  if (!f.read(magic, 4) || std::memcmp(magic, kMagic, 4) != 0)
    throw StepError(file + ": invalid file format");
  if (get<int32_t>(f, file) > kBinaryVersion)
    throw StepError(file + ": incompatible file format version");
  if (!f.read(type, 4)) throw StepError(file + ": truncated");
  const int32_t bytes = get<int32_t>(f, file), per = get<int32_t>(f, file);
  const int32_t order = get<int32_t>(f, file);
  get<int32_t>(f, file);
  get<int32_t>(f, file);
  if (bytes != (complex ? 16 : 8) || per != (complex ? 2 : 1))
    throw StepError(file + ": holds a " + (per == 2 ? "complex" : "real") +
                    " tensor; set complexVersion accordingly");
  if (order < 0 || order > 16) throw StepError(file + ": bad order");
  auto t = std::make_shared<HTensor>();
  int64_t n = 1;
  for (int d = 0; d < order; ++d) {
    const int32_t len = get<int32_t>(f, file);
    get<char>(f, file);
    get<int8_t>(f, file);
    get<int16_t>(f, file);
    if (len < 0 || (len > 0 && n > (INT64_MAX / 16) / len)) throw StepError(file + ": bad length");
    n *= len;
    t->lens.push_back(len);
  }
  t->complex = complex;
  t->re.resize(n);
  if (complex) t->im.resize(n);
  for (int64_t e = 0; e < n; ++e) {
    t->re[e] = get<double>(f, file);
    if (complex) t->im[e] = get<double>(f, file);
  }
  return t;
}

void write_tensor_text(const std::string &file, const std::string &name, const HTensor &t,
                       std::string rows, const std::string &cols, const std::string &delim) {
  const int order = (int)t.lens.size();
  if (rows.empty() && cols.empty())
    for (int d = 0; d < order; ++d) rows += (char)('i' + d);
  int64_t ncols = 1;
  const std::vector<int64_t> off = text_layout(t, rows, cols, &ncols);
  std::ofstream f(file);
  if (!f) throw StepError("cannot open " + file);
  f << name << delim << order;
  for (auto l : t.lens) f << delim << l;
  f << "\n" << rows << delim << cols << "\n";
  f << std::setprecision(16);
  auto value = [&](int64_t e) {
    if (t.complex) f << std::complex<double>(t.re[off[e]], t.im[off[e]]);
    else f << t.re[off[e]];
  };
  for (int64_t e = 0; e < t.size(); e += ncols) {
    value(e);
    for (int64_t c = 1; c < ncols; ++c) {
      f << delim;
      value(e + c);
    }
    f << "\n";
  }
}

std::shared_ptr<HTensor> read_tensor_text(const std::string &file, bool complex) {
  std::ifstream f(file);
  if (!f) throw StepError("Failed to open file \"" + file + "\"");
  std::string line, rows, cols;
  std::getline(f, line);
  const size_t sp = line.find(' ');
  std::istringstream head(sp == std::string::npos ? "" : line.substr(sp + 1));
  int order = -1;
  head >> order;
  if (order < 0 || order > 16) throw StepError(file + ": bad header");
  auto t = std::make_shared<HTensor>();
  for (int d = 0; d < order; ++d) {
    long long l = -1;
    head >> l;
    if (l < 0) throw StepError(file + ": bad header");
    t->lens.push_back(l);
  }
  std::getline(f, line);
  const size_t sp2 = line.find(' ');
  rows = line.substr(0, sp2);
  cols = sp2 == std::string::npos ? "" : line.substr(sp2 + 1);
  while (!cols.empty() && (cols.back() == '\r' || cols.back() == ' ')) cols.pop_back();
  t->complex = complex;
  t->re.assign((size_t)t->size(), 0.0);
  if (complex) t->im.assign((size_t)t->size(), 0.0);
  int64_t ncols = 1;
  const std::vector<int64_t> off = text_layout(*t, rows, cols, &ncols);
  // numbers as the reference's NumberScanner reads them (strtod; complex as
  // "(re,im)"), skipping anything between them
  std::stringstream ss;
  ss << f.rdbuf();
  const std::string body = ss.str();
  const char *p = body.c_str();
  auto number = [&]() {
    while (*p && !(std::isdigit((unsigned char)*p) || *p == '-' || *p == '+' || *p == '.'))
      ++p;
    char *end = nullptr;
    const double v = std::strtod(p, &end);
    if (end == p) throw StepError(file + ": too few elements");
    p = end;
    return v;
  };
  for (int64_t e = 0; e < t->size(); ++e) {
    t->re[off[e]] = number();
    if (complex) t->im[off[e]] = number();
  }
  return t;
}

// TensorWriter (src/algorithms/TensorWriter.cxx:21-81)
struct TensorWriter : Algorithm {
  void run() override {
    auto d = arg("Data");
    const bool binary = text("mode", "text") == "binary";
    const std::string file = text("file", d->name + (binary ? ".bin" : ".dat"));
    const HTensor &t = tensor("Data");
    if (binary) write_tensor_binary(file, t);
    else write_tensor_text(file, d->name, t, text("rowIndexOrder", ""),
                           text("columnIndexOrder", ""), text("delimiter", " "));
    emit["Data"] = d->name;
    emit["file"] = file;
    emit["elements"] = (long long)t.size();
  }
};
REGISTER_ALGORITHM(TensorWriter);

// TensorReader (src/algorithms/TensorReader.cxx:14-63)
struct TensorReader : Algorithm {
  void run() override {
    auto d = arg("Data");
    const bool binary = text("mode", "text") == "binary";
    const bool complex = integer("complexVersion", 0) == 1;
    if (integer("precision", 64) != 64) throw StepError("only precision 64 is supported");
    const std::string file = text("file", d->name + (binary ? ".bin" : ".dat"));
    auto t = binary ? read_tensor_binary(file, complex) : read_tensor_text(file, complex);
    emit["file"] = file;
    emit["Data"] = d->name;
    emit["elements"] = (long long)t->size();
    set_tensor("Data", t);
  }
};
REGISTER_ALGORITHM(TensorReader);

// DefineHolesAndParticles (src/algorithms/cc4s/DefineHolesAndParticles.cxx:8-51)
struct DefineHolesAndParticles : Algorithm {
  void run() override {
    auto h = yl::parse_file(text("fileName"));
    auto md = h->get("metaData");
    if (!md || !md->get("fermiEnergy") || !md->get("energies"))
      throw StepError("metaData.fermiEnergy / metaData.energies missing");
    const double ef = md->get("fermiEnergy")->as_double();
    std::vector<double> e;
    for (auto &x : md->get("energies")->seq) e.push_back(x->as_double());
    auto it = std::stable_partition(e.begin(), e.end(), [&](double v) { return v <= ef; });
    auto ho = std::make_shared<HTensor>(), pa = std::make_shared<HTensor>();
    ho->re.assign(e.begin(), it);
    pa->re.assign(it, e.end());
    ho->lens = {(int64_t)ho->re.size()};
    pa->lens = {(int64_t)pa->re.size()};
    emit["No"] = (long long)ho->re.size();
    emit["Nv"] = (long long)pa->re.size();
    set_tensor("HoleEigenEnergies", ho);
    set_tensor("ParticleEigenEnergies", pa);
  }
};
REGISTER_ALGORITHM(DefineHolesAndParticles);

struct Sizes {
  int No, Nv, NG;
};

Sizes sizes_of(const Algorithm &a) {
  const HTensor &eh = a.tensor("HoleEigenEnergies");
  const HTensor &ep = a.tensor("ParticleEigenEnergies");
  if (eh.lens.size() != 1 || ep.lens.size() != 1)
    throw StepError("HoleEigenEnergies and ParticleEigenEnergies must be vectors");
  if (eh.lens[0] < 1 || ep.lens[0] < 1 || eh.lens[0] + ep.lens[0] > (1 << 20))
    throw StepError("No and Nv must be positive and No+Nv at most 2^20");
  Sizes s{(int)eh.lens[0], (int)ep.lens[0], 0};
  if (a.given("CoulombVertex")) {
    const HTensor &g = a.tensor("CoulombVertex");
    if (g.lens.size() != 3 || g.lens[1] != s.No + s.Nv || g.lens[2] != s.No + s.Nv)
      throw StepError("CoulombVertex must be [NG, No+Nv, No+Nv]");
    if (g.lens[0] < 1 || g.lens[0] > INT32_MAX) throw StepError("CoulombVertex: bad NG");
    s.NG = (int)g.lens[0];
  }
  return s;
}

bool has_imaginary_part(const HTensor &t) {
  if (!t.complex) return false;
  for (double v : t.im)
    if (v != 0.0) return true;
  return false;
}

// interleaved (re, im) copy of a tensor, as CTF stores complex<double>
std::vector<double> interleaved(const HTensor &t) {
  std::vector<double> z(2 * (size_t)t.size(), 0.0);
  for (int64_t e = 0; e < t.size(); ++e) {
    z[2 * e] = t.re[e];
    if (t.complex) z[2 * e + 1] = t.im[e];
  }
  return z;
}

// The real path reads a complex vertex as Re.Re + Im.Im in every product of
// two vertex factors (CcsdEnergyFromCoulombIntegrals.cxx:80-115,162-169,...;
// CcsdPerturbativeTriplesComplex.cxx:330-341): that is the real vertex with
// the imaginary rows stacked under the real ones, [Re; Im] of 2 NG rows.
const double *real_vertex(const HTensor &g, int *NG, std::vector<double> &buf) {
  if (!has_imaginary_part(g)) return g.re.data();
  const int64_t G = g.lens[0], pq = g.size() / G;
  buf.resize(2 * (size_t)g.size());
  for (int64_t e = 0; e < pq; ++e)
    for (int64_t r = 0; r < G; ++r) {
      buf[r + 2 * G * e] = g.re[r + G * e];
      buf[G + r + 2 * G * e] = g.im[r + G * e];
    }
  *NG = (int)(2 * G);
  return buf.data();
}

// the reference takes its complex branch when the PPHH integrals are complex
// (ClusterSinglesDoublesAlgorithm.cxx:25-35, CcsdPerturbativeTriplesComplex.cxx:50-80)
bool complex_integrals_given(const HTensor *pphh) { return pphh && pphh->complex; }

std::shared_ptr<HTensor> complex_tensor(const std::vector<int64_t> &lens,
                                        const std::vector<double> &z) {
  auto t = std::make_shared<HTensor>();
  t->lens = lens;
  t->complex = true;
  t->re.resize(t->size());
  t->im.resize(t->size());
  for (int64_t e = 0; e < t->size(); ++e) {
    t->re[e] = z[2 * e];
    t->im[e] = z[2 * e + 1];
  }
  return t;
}

// CoulombIntegralsFromVertex, real integrals (CoulombIntegralsFromVertex.cxx:203-558)
struct CoulombIntegralsFromVertex : Algorithm {
  // complex: 1, calculateComplexIntegrals (CoulombIntegralsFromVertex.cxx:613-816)
  void run_complex() {
    const Sizes s = sizes_of(*this);
    const std::vector<double> gz = interleaved(tensor("CoulombVertex"));
    const int64_t o = s.No, v = s.Nv;
    const std::pair<const char *, std::vector<int64_t>> blocks[7] = {
        {"PPHHCoulombIntegrals", {v, v, o, o}}, {"PHHPCoulombIntegrals", {v, o, o, v}},
        {"HHPPCoulombIntegrals", {o, o, v, v}}, {"PHPHCoulombIntegrals", {v, o, v, o}},
        {"HHHHCoulombIntegrals", {o, o, o, o}}, {"HHHPCoulombIntegrals", {o, o, o, v}},
        {"PHHHCoulombIntegrals", {v, o, o, o}}};
    std::vector<std::vector<double>> bufs(7);
    double *out[7];
    for (int q = 0; q < 7; ++q) {
      out[q] = nullptr;
      if (!given(blocks[q].first)) continue;
      size_t n = 2;
      for (auto l : blocks[q].second) n *= (size_t)l;
      bufs[q].assign(n, 0.0);
      out[q] = bufs[q].data();
    }
    check(gbcc_coulomb_integrals_complex(gpu(), s.No, s.Nv, s.NG, gz.data(), out[0], out[1],
                                         out[2], out[3], out[4], out[5], out[6]),
          "CoulombIntegralsFromVertex");
    Json list = Json::array();
    for (int q = 0; q < 7; ++q)
      if (out[q]) {
        set_tensor(blocks[q].first, complex_tensor(blocks[q].second, bufs[q]));
        list.push(blocks[q].first);
      }
    for (auto &a : args)
      if (a.first.find("CoulombIntegrals") != std::string::npos) {
        bool ok = false;
        for (auto &b : blocks) ok |= a.first == b.first;
        if (!ok)
          log(0, "CoulombIntegralsFromVertex",
              "WARNING: " + a.first + " is not built (not used by the complex CCSD/(T))");
      }
    emit["NG"] = s.NG;
    emit["No"] = s.No;
    emit["Nv"] = s.Nv;
    emit["complex"] = 1;
    emit["integrals"] = list;
  }

  void run() override {
    if (integer("antisymmetrize", 0))
      throw StepError("antisymmetrized integrals are not supported");
    if (integer("complex", 0)) {
      run_complex();
      return;
    }
    Sizes s = sizes_of(*this);
    std::vector<double> stacked;
    const double *gre = real_vertex(tensor("CoulombVertex"), &s.NG, stacked);
    const int64_t o = s.No, v = s.Nv;
    auto mk = [&](std::initializer_list<int64_t> l) {
      auto t = std::make_shared<HTensor>();
      t->lens = l;
      t->re.resize(t->size());
      return t;
    };
    std::shared_ptr<HTensor> pphh = mk({v, v, o, o}), phph = mk({v, o, v, o}),
                             hhhh = mk({o, o, o, o}), hhhp = mk({o, o, o, v}),
                             hhpp = mk({o, o, v, v});
    check(gbcc_coulomb_integrals(gpu(), s.No, s.Nv, s.NG, gre,
                                 pphh->re.data(), phph->re.data(), hhhh->re.data(),
                                 hhhp->re.data(), hhpp->re.data()),
          "CoulombIntegralsFromVertex");
    // the particle blocks of the stored formulation, only when requested
    // (PPPP alone is Nv^4 doubles)
    std::shared_ptr<HTensor> pppp, ppph;
    if (given("PPPPCoulombIntegrals") || given("PPPHCoulombIntegrals")) {
      if (given("PPPPCoulombIntegrals")) pppp = mk({v, v, v, v});
      if (given("PPPHCoulombIntegrals")) ppph = mk({v, v, v, o});
      check(gbcc_coulomb_integrals_pp(gpu(), s.No, s.Nv, s.NG, gre,
                                      pppp ? pppp->re.data() : nullptr,
                                      ppph ? ppph->re.data() : nullptr),
            "CoulombIntegralsFromVertex");
    }
    Json list = Json::array();
    const std::pair<const char *, std::shared_ptr<HTensor>> built[] = {
        {"PPHHCoulombIntegrals", pphh}, {"PHPHCoulombIntegrals", phph},
        {"HHHHCoulombIntegrals", hhhh}, {"HHHPCoulombIntegrals", hhhp},
        {"HHPPCoulombIntegrals", hhpp}, {"PPPPCoulombIntegrals", pppp},
        {"PPPHCoulombIntegrals", ppph}};
    for (auto &b : built)
      if (given(b.first)) {
        set_tensor(b.first, b.second);
        list.push(b.first);
      }
    for (auto &a : args)
      if (a.first.find("CoulombIntegrals") != std::string::npos) {
        bool ok = false;
        for (auto &b : built) ok |= a.first == b.first;
        if (!ok)
          log(0, "CoulombIntegralsFromVertex",
              "WARNING: " + a.first + " is not built (not used by CCSD/(T))");
      }
    emit["NG"] = s.NG;
    emit["No"] = s.No;
    emit["Nv"] = s.Nv;
    emit["integrals"] = list;
  }
};
REGISTER_ALGORITHM(CoulombIntegralsFromVertex);

int precision_of(const Algorithm &a) {
  const std::string p = a.text("precision", "fp64");
  if (p == "fp64") return GBCC_PREC_FP64;
  if (p == "emu" || p == "mixed") return GBCC_PREC_EMU;
  throw StepError("precision must be fp64 or emu");
}

// CcsdEnergyFromCoulombIntegrals (ClusterSinglesDoublesAlgorithm.cxx:25-128)
struct CcsdEnergyFromCoulombIntegrals : Algorithm {
  // 0: particle ladder from the vertex; 1: stored Vabcd / Vabci
  // (CcsdEnergyFromCoulombIntegralsReference)
  virtual int formulation() const { return 0; }

  // the complex branch, taken when the vertex is complex (:25-35); the
  // integrals are built from the vertex on the device
  void run_complex(const Sizes &s, const gbcc_ccsd_opts &o) {
    const int64_t o1 = s.No, v1 = s.Nv;
    const std::vector<double> g = interleaved(tensor("CoulombVertex"));
    std::vector<double> t1i, t2i;
    gbcc_ccsd_complex_in in{};
    in.No = s.No; in.Nv = s.Nv; in.NG = s.NG;
    in.eps_h = tensor("HoleEigenEnergies").re.data();
    in.eps_p = tensor("ParticleEigenEnergies").re.data();
    in.gamma = g.data();
    if (given("initialSinglesAmplitudes")) {
      t1i = interleaved(tensor("initialSinglesAmplitudes", {v1, o1}));
      in.init_T1 = t1i.data();
    }
    if (given("initialDoublesAmplitudes")) {
      t2i = interleaved(tensor("initialDoublesAmplitudes", {v1, v1, o1, o1}));
      in.init_T2 = t2i.data();
    }
    std::vector<double> fi;
    if (given("HPFockMatrix")) {
      fi = interleaved(tensor("HPFockMatrix", {o1, v1}));
      in.fock_hp = fi.data();
    }
    std::vector<double> t1(2 * v1 * o1), t2(2 * v1 * v1 * o1 * o1);
    std::vector<double> hist(2 * std::max(o.max_iterations, 1)), pe(2 * o1 * o1);
    gbcc_ccsd_complex_out out{};
    out.T1 = t1.data();
    out.T2 = t2.data();
    out.energy_history = hist.data();
    out.pair_energy = given("PairEnergy") ? pe.data() : nullptr;
    emit["complex"] = 1;
    const gbcc_status st = gbcc_ccsd_solve_complex(gpu(), &in, &o, &out);
    check(st, "CcsdEnergyFromCoulombIntegrals (complex)", true);
    Json its = Json::array();
    for (int i = 0; i < out.iterations; ++i) {
      Json it = Json::object();
      it["iteration"] = i + 1;
      it["energy"]["value"] = hist[2 * i];
      its.push(it);
    }
    emit["iterations"] = its;
    const double d = out.direct[0], x = out.exchange[0];       // real parts (:190-196)
    emit["energy"]["direct"] = d;
    emit["energy"]["exchange"] = x;
    emit["energy"]["singlet"] = 0.25 * d - 0.5 * x;
    emit["energy"]["triplet"] = 0.75 * d + 1.5 * x;
    emit["energy"]["value"] = out.energy[0];
    emit["energy"]["imaginary"] = out.energy[1];
    emit["convergenceReached"] = out.converged;
    if (st == GBCC_NOT_CONVERGED)
      log(0, "CCSD", "WARNING: energy or amplitudes convergence not reached.");
    std::ostringstream m;
    m << std::setprecision(10) << "energy= " << out.energy[0];
    log(0, "CCSD", m.str());
    set_real("CcsdEnergy", out.energy[0]);                      // std::real (:32)
    if (given("CcsdSinglesAmplitudes"))
      set_tensor("CcsdSinglesAmplitudes", complex_tensor({v1, o1}, t1));
    if (given("CcsdDoublesAmplitudes"))
      set_tensor("CcsdDoublesAmplitudes", complex_tensor({v1, v1, o1, o1}, t2));
    if (given("PairEnergy")) set_tensor("PairEnergy", complex_tensor({o1, o1}, pe));
  }

  void run() override {
    const Sizes s = sizes_of(*this);
    if (formulation() == 0 && !given("CoulombVertex"))
      throw StepError("CoulombVertex is required");
    gbcc_ccsd_opts o;
    gbcc_ccsd_opts_default(&o);
    o.formulation = formulation();
    if (formulation() == 1) o.only_ppl = (int)integer("onlyPPL", 0);
    const std::string mixer = text("mixer", "LinearMixer");
    if (mixer == "LinearMixer") o.mixer = 0;
    else if (mixer == "DiisMixer") o.mixer = 1;
    else throw StepError("Mixer not implemented: " + mixer);
    o.max_residua = (int)real("maxResidua", 4);  // DiisMixer.cxx:55 reads it as real
    o.mixing_ratio = real("mixingRatio", 1.0);
    o.max_iterations = (int)integer("maxIterations", 16);
    o.energy_convergence = real("energyConvergence", 1e-6);
    o.amplitudes_convergence = real("amplitudesConvergence", 1e-5);
    o.level_shift = real("levelShift", 0.0);
    o.distinguishable = (int)integer("distinguishable", 0);
    o.ppl = (int)integer("ppl", 1);
    o.integrals_slice_size = (int)integer("integralsSliceSize", -1);
    o.integrals_slice_factor = given("integralsSliceFactor") ? real("integralsSliceFactor") : -1.0;
    o.precision = precision_of(*this);
    o.emu_slices = (int)integer("emulationDigits", 0);
    if (integer("unrestricted", 0) || integer("antisymmetrize", 0))
      throw StepError("unrestricted / antisymmetrized amplitudes are not supported");
    emit["maxIterations"] = o.max_iterations;                     // :65-70
    emit["amplitudesConvergence"] = std::abs(o.amplitudes_convergence);
    emit["energyConvergence"] = std::abs(o.energy_convergence);
    for (const char *k : {"distinguishable", "PPL", "OnlyPPL", "integralsSliceSize"})  // :72-87
      if (given(k)) emit[k] = integer(k, 0);
    emit["precision"] = o.precision == GBCC_PREC_FP64 ? "fp64" : "emu";
    if (complex_integrals_given(given("PPHHCoulombIntegrals") ? &tensor("PPHHCoulombIntegrals")
                                                              : nullptr)) {
      if (formulation() != 0)
        throw StepError("only CcsdEnergyFromCoulombIntegrals has a complex branch here");
      if (!given("CoulombVertex")) throw StepError("CoulombVertex is required");
      run_complex(s, o);
      return;
    }
    gbcc_ccsd_in in{};
    in.No = s.No; in.Nv = s.Nv; in.NG = s.NG;
    in.eps_h = tensor("HoleEigenEnergies").re.data();
    in.eps_p = tensor("ParticleEigenEnergies").re.data();
    std::vector<double> stacked;
    if (given("CoulombVertex")) in.gamma = real_vertex(tensor("CoulombVertex"), &in.NG, stacked);
    const int64_t o1 = s.No, v1 = s.Nv;
    if (formulation() == 1) {
      in.Vabcd = tensor_or_null("PPPPCoulombIntegrals", {v1, v1, v1, v1});
      in.Vabci = tensor_or_null("PPPHCoulombIntegrals", {v1, v1, v1, o1});
    }
    in.Vabij = tensor_or_null("PPHHCoulombIntegrals", {v1, v1, o1, o1});
    in.Vaibj = tensor_or_null("PHPHCoulombIntegrals", {v1, o1, v1, o1});
    in.Vijkl = tensor_or_null("HHHHCoulombIntegrals", {o1, o1, o1, o1});
    in.Vijka = tensor_or_null("HHHPCoulombIntegrals", {o1, o1, o1, v1});
    in.init_T1 = tensor_or_null("initialSinglesAmplitudes", {v1, o1});
    in.init_T2 = tensor_or_null("initialDoublesAmplitudes", {v1, v1, o1, o1});
    in.fock_hp = tensor_or_null("HPFockMatrix", {o1, v1});
    auto t1 = std::make_shared<HTensor>(), t2 = std::make_shared<HTensor>(),
         pe = std::make_shared<HTensor>();
    t1->lens = {v1, o1};
    t2->lens = {v1, v1, o1, o1};
    pe->lens = {o1, o1};
    t1->re.resize(t1->size());
    t2->re.resize(t2->size());
    pe->re.resize(pe->size());
    std::vector<double> hist(std::max(o.max_iterations, 1));
    gbcc_ccsd_out out{};
    out.T1 = t1->re.data();
    out.T2 = t2->re.data();
    out.pair_energy = given("PairEnergy") ? pe->re.data() : nullptr;
    out.energy_history = hist.data();
    gbcc_status st = gbcc_ccsd_solve(gpu(), &in, &o, &out);
    check(st, "CcsdEnergyFromCoulombIntegrals", true);
    Json its = Json::array();
    for (int i = 0; i < out.iterations; ++i) {
      Json it = Json::object();
      it["iteration"] = i + 1;
      it["energy"]["value"] = hist[i];
      its.push(it);
    }
    emit["iterations"] = its;
    const double d = out.direct, x = out.exchange;
    emit["energy"]["direct"] = d;
    emit["energy"]["exchange"] = x;
    emit["energy"]["singlet"] = 0.25 * d - 0.5 * x;
    emit["energy"]["triplet"] = 0.75 * d + 1.5 * x;
    emit["energy"]["value"] = out.energy;
    emit["convergenceReached"] = out.converged;
    if (st == GBCC_NOT_CONVERGED)
      log(0, "CCSD", "WARNING: energy or amplitudes convergence not reached.");
    std::ostringstream m;
    m << std::setprecision(10) << "energy= " << out.energy;
    log(0, "CCSD", m.str());
    set_real("CcsdEnergy", out.energy);
    if (given("CcsdSinglesAmplitudes")) set_tensor("CcsdSinglesAmplitudes", t1);
    if (given("CcsdDoublesAmplitudes")) set_tensor("CcsdDoublesAmplitudes", t2);
    if (given("PairEnergy")) set_tensor("PairEnergy", pe);
  }
};
REGISTER_ALGORITHM(CcsdEnergyFromCoulombIntegrals);

// CcsdEnergyFromCoulombIntegralsReference
// (src/algorithms/CcsdEnergyFromCoulombIntegralsReference.cxx:29-292): the
// same driver and outputs, with the ladder from resident PPPP / PPPH
// integrals; the vertex is optional when every integral is given.
struct CcsdEnergyFromCoulombIntegralsReference : CcsdEnergyFromCoulombIntegrals {
  int formulation() const override { return 1; }
};
REGISTER_ALGORITHM(CcsdEnergyFromCoulombIntegralsReference);

// CcsdPerturbativeTriples (CcsdPerturbativeTriples.cxx:119-248)
struct CcsdPerturbativeTriples : Algorithm {
  void run() override {
    const Sizes s = sizes_of(*this);
    if (!given("CoulombVertex")) throw StepError("CoulombVertex is required");
    gbcc_triples_in in{};
    in.No = s.No; in.Nv = s.Nv; in.NG = s.NG;
    in.eps_h = tensor("HoleEigenEnergies").re.data();
    in.eps_p = tensor("ParticleEigenEnergies").re.data();
    std::vector<double> stacked;
    in.gamma = real_vertex(tensor("CoulombVertex"), &in.NG, stacked);
    const int64_t o1 = s.No, v1 = s.Nv;
    in.Vabij = tensor_or_null("PPHHCoulombIntegrals", {v1, v1, o1, o1});
    in.Vijka = tensor_or_null("HHHPCoulombIntegrals", {o1, o1, o1, v1});
    const HTensor &t1 = tensor("CcsdSinglesAmplitudes", {v1, o1});
    const HTensor &t2 = tensor("CcsdDoublesAmplitudes", {v1, v1, o1, o1});
    if (has_imaginary_part(t1) || has_imaginary_part(t2))
      throw StepError("complex amplitudes: use CcsdPerturbativeTriplesComplex, the reference's "
                      "(T) for complex amplitudes");
    in.T1 = t1.re.data();
    in.T2 = t2.re.data();
    in.e_ccsd = real("CcsdEnergy");
    double etot = 0, et = 0;
    check(gbcc_triples(gpu(), &in, precision_of(*this), &etot, &et),
          "CcsdPerturbativeTriples");
    std::ostringstream m;
    m << std::setprecision(12) << "e=" << etot << " triples=" << et;
    log(0, "CcsdPerturbativeTriples", m.str());
    emit["energy"]["triples"] = et;
    emit["energy"]["value"] = etot;
    set_real("CcsdPerturbativeTriplesEnergy", etot);
  }
};
REGISTER_ALGORITHM(CcsdPerturbativeTriples);

// CcsdPerturbativeTriplesComplex (CcsdPerturbativeTriplesComplex.cxx:32-84):
// complex amplitudes go through the complex Calculator; real amplitudes with a
// real vertex are the real (T).  The PPHH / PHHH integrals are built from the
// vertex on the device.
struct CcsdPerturbativeTriplesComplex : Algorithm {
  void run() override {
    const Sizes s = sizes_of(*this);
    if (!given("CoulombVertex")) throw StepError("CoulombVertex is required");
    const int64_t o1 = s.No, v1 = s.Nv;
    const HTensor &g = tensor("CoulombVertex");
    const HTensor &t1 = tensor("CcsdSinglesAmplitudes", {v1, o1});
    const HTensor &t2 = tensor("CcsdDoublesAmplitudes", {v1, v1, o1, o1});
    const double e_ccsd = real("CcsdEnergy");
    double etot = 0, et[2] = {0, 0};
    // Calculator<complex> for complex integrals (:50-80); without integrals,
    // for complex amplitudes
    const bool cplx = given("PPHHCoulombIntegrals")
                          ? complex_integrals_given(&tensor("PPHHCoulombIntegrals"))
                          : (t1.complex || t2.complex);
    if (cplx) {
      const std::vector<double> gz = interleaved(g), t1z = interleaved(t1),
                                t2z = interleaved(t2);
      gbcc_triples_complex_in in{};
      in.No = s.No; in.Nv = s.Nv; in.NG = s.NG;
      in.eps_h = tensor("HoleEigenEnergies").re.data();
      in.eps_p = tensor("ParticleEigenEnergies").re.data();
      in.gamma = gz.data();
      in.T1 = t1z.data();
      in.T2 = t2z.data();
      in.e_ccsd = e_ccsd;
      check(gbcc_triples_complex(gpu(), &in, precision_of(*this), &etot, et),
            "CcsdPerturbativeTriplesComplex");
    } else {
      if (has_imaginary_part(t1) || has_imaginary_part(t2))
        throw StepError("complex amplitudes with real integrals");
      gbcc_triples_in in{};
      in.No = s.No; in.Nv = s.Nv; in.NG = s.NG;
      in.eps_h = tensor("HoleEigenEnergies").re.data();
      in.eps_p = tensor("ParticleEigenEnergies").re.data();
      std::vector<double> stacked;
      in.gamma = real_vertex(g, &in.NG, stacked);  // Calculator<double> (:330-341)
      in.T1 = t1.re.data();
      in.T2 = t2.re.data();
      in.e_ccsd = e_ccsd;
      check(gbcc_triples(gpu(), &in, precision_of(*this), &etot, et),
            "CcsdPerturbativeTriplesComplex");
    }
    std::ostringstream m;
    m << std::setprecision(12) << "e=" << etot << " triples=" << et[0];
    log(0, "CcsdPerturbativeTriplesComplex", m.str());
    emit["energy"]["triples"] = et[0];
    emit["energy"]["triplesImaginary"] = et[1];
    emit["energy"]["value"] = etot;
    set_real("CcsdPerturbativeTriplesComplexEnergy", etot);       // :84
  }
};
REGISTER_ALGORITHM(CcsdPerturbativeTriplesComplex);

// ------------------------------------------------------------------ parser
std::vector<std::unique_ptr<Algorithm>> parse_steps(const std::string &file) {
  auto doc = yl::parse_file(file);
  if (!doc->is_seq()) throw StepError("input file must be a list of steps");
  std::vector<std::unique_ptr<Algorithm>> algs;
  for (auto &node : doc->seq) {
    if (!node->is_map() || !node->get("name"))
      throw StepError("every step needs a name");
    const std::string name = node->get("name")->str();
    if (node->get("disable") && node->get("disable")->as_bool()) continue;
    if (node->get("enable") && !node->get("enable")->as_bool()) continue;
    auto f = registry().find(name);
    if (f == registry().end()) throw StepError("unknown algorithm " + name);
    auto a = f->second();
    a->name = name;
    for (const char *io : {"in", "out"}) {
      auto m = node->get(io);
      if (!m || m->kind == yl::Node::Null) continue;
      if (!m->is_map()) throw StepError(std::string(io) + " of " + name + " must be a map");
      for (auto &kv : m->map) {
        if (!kv.second->is_scalar())
          throw StepError("argument " + kv.first + " of " + name + " must be a scalar");
        const std::string &v = kv.second->scalar;
        long long iv;
        double dv;
        std::string dn;
        if (!kv.second->quoted && yl::scalar_is_int(v, &iv)) {
          auto d = anon(Data::Integer);
          d->integer = iv;
          dn = d->name;
        } else if (!kv.second->quoted && yl::scalar_is_double(v, &dv)) {
          auto d = anon(Data::Real);
          d->real = dv;
          dn = d->name;
        } else if (!v.empty() && v[0] == '$') {
          dn = data_symbol(v.substr(1))->name;
        } else {
          auto d = anon(Data::Text);
          d->text = v;
          dn = d->name;
        }
        a->args.emplace_back(kv.first, dn);
      }
    }
    if (node->get("note")) a->note = node->get("note")->str();
    if (node->get("fallible")) a->fallible = node->get("fallible")->as_bool();
    algs.push_back(std::move(a));
  }
  return algs;
}

Json args_json(const Algorithm &a, bool out) {
  Json j = Json::object();
  (void)out;
  for (auto &kv : a.args) {
    auto d = data_symbol(kv.second);
    switch (d->kind) {
      case Data::Integer: j[kv.first] = d->integer; break;
      case Data::Real: j[kv.first] = d->real; break;
      case Data::Text: j[kv.first] = d->text; break;
      default: j[kv.first] = d->name; break;
    }
  }
  return j;
}

void usage() {
  std::cout << "usage: sisi4s-gb300 -i INPUT.yaml [-o OUT.yaml] [-l LOG] [--dry] "
               "[--log-level N] [--list]\n";
}

}  // namespace

int main(int argc, char **argv) {
  std::string in, out = "sisi4s.out.yaml", logf = "sisi4s.log";
  bool dry = false, list = false;
  for (int i = 1; i < argc; ++i) {
    const std::string a = argv[i];
    auto next = [&]() -> std::string {
      if (i + 1 >= argc) { usage(); std::exit(2); }
      return argv[++i];
    };
    if (a == "-i" || a == "--in") in = next();
    else if (a == "-o" || a == "--out") out = next();
    else if (a == "-l" || a == "--log") logf = next();
    else if (a == "--dry") dry = true;
    else if (a == "--log-level") g_log_level = std::atoi(next().c_str());
    else if (a == "--list" || a == "--list-algorithms") list = true;
    else if (a == "-h" || a == "--help") { usage(); return 0; }
    else { usage(); return 2; }
  }
  if (list) {
    for (auto &kv : registry()) std::cout << kv.first << "\n";
    return 0;
  }
  if (in.empty()) { usage(); return 2; }
  g_log.open(logf);
  Json root = Json::object();
  root["version"] = "sisi4s-gb300";
  root["abi"] = gbcc_abi_version();
  root["dryRun"] = dry ? 1 : 0;
  Json steps = Json::array();
  int rc = 0;
  try {
    auto algs = parse_steps(in);
    for (size_t i = 0; i < algs.size(); ++i) {
      Algorithm &a = *algs[i];
      Json st = Json::object();
      st["name"] = a.name;
      if (!a.note.empty()) st["note"] = a.note;
      st["in"] = args_json(a, false);
      log(0, "root", "step: " + std::to_string(i + 1) + ", " + a.name);
      const auto t0 = std::chrono::steady_clock::now();
      if (!dry) {
        try {
          a.run();
        } catch (const std::exception &e) {
          if (!a.fallible) throw;
          log(0, "root", std::string("fallible step failed: ") + e.what());
          st["failed"] = e.what();
        }
      }
      const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      for (auto &kv : a.emit.obj) st[kv.first] = kv.second;
      st["out"] = args_json(a, true);
      st["realtime"] = dt;
      steps.push(st);
    }
  } catch (const std::exception &e) {
    std::cerr << "error: " << e.what() << std::endl;
    if (g_log) g_log << "error: " << e.what() << std::endl;
    root["error"] = e.what();
    rc = 1;
  }
  root["steps"] = steps;
  std::ofstream o(out);
  root.dump(o);
  o << "\n";
  if (g_ctx) gbcc_ctx_destroy(g_ctx);
  return rc;
}
