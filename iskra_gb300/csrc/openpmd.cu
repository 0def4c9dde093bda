// openpmd.cu -- openPMD records of one iteration written as an HDF5 file,
// the diagnostics of Diagnostics/src/hdf5.jl (new_iteration :47-66,
// save_record :69-101) with the metadata of Diagnostics/src/openpmd/*.jl.
//
// No HDF5 library is linked: the file is laid out directly from the
// published HDF5 file format (version 2 superblock, version 2 object
// headers, groups in compact link storage, contiguous datasets, version 3
// attribute messages, Jenkins lookup3 checksums).  The file holds, under
// /data/<iteration>/ (openPMD base path "/data/%T", file-based encoding
// "data%T.h5" in <prefix>/hdf5/):
//   fields/rho, fields/phi, fields/E/{x,y,z}, fields/n<species>,
//   fields/nuMCC-<species>-<k> (accepted collisions per node of process k
//     since the previous record),
//   fields/{Q1, I1, V1, Vext} (the RLC circuit's charge, current, source and
//     device voltage, when a circuit is attached),
//   particles/<species>/{position/{x,y}, momentum/{x,y,z}, weighting, id,
//     charge, mass, positionOffset/{x,y,z}},
// with the reference's attributes (unitDimension, unitSI, gridSpacing, ...).
// Field arrays keep Julia's memory order (x fastest), i.e. HDF5 dimensions
// (ny, nx), as HDF5.jl writes a Julia (nx, ny) array.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "internal.cuh"

namespace iskra {

// ---- Jenkins lookup3 hashlittle (Bob Jenkins, 2006, public domain), the
// checksum of HDF5 metadata blocks ---------------------------------------
static inline uint32_t rot32(uint32_t x, int k) { return (x << k) | (x >> (32 - k)); }

static uint32_t lookup3(const uint8_t *k, size_t length, uint32_t initval) {
  uint32_t a, b, c;
  a = b = c = 0xdeadbeefu + (uint32_t)length + initval;
  auto le = [](const uint8_t *p) {
    return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
  };
  while (length > 12) {
    a += le(k);
    b += le(k + 4);
    c += le(k + 8);
    a -= c; a ^= rot32(c, 4);  c += b;
    b -= a; b ^= rot32(a, 6);  a += c;
    c -= b; c ^= rot32(b, 8);  b += a;
    a -= c; a ^= rot32(c, 16); c += b;
    b -= a; b ^= rot32(a, 19); a += c;
    c -= b; c ^= rot32(b, 4);  b += a;
    length -= 12;
    k += 12;
  }
  switch (length) {  // the last block, fall-through
    case 12: c += (uint32_t)k[11] << 24;  // fall through
    case 11: c += (uint32_t)k[10] << 16;  // fall through
    case 10: c += (uint32_t)k[9] << 8;    // fall through
    case 9: c += k[8];                    // fall through
    case 8: b += (uint32_t)k[7] << 24;    // fall through
    case 7: b += (uint32_t)k[6] << 16;    // fall through
    case 6: b += (uint32_t)k[5] << 8;     // fall through
    case 5: b += k[4];                    // fall through
    case 4: a += (uint32_t)k[3] << 24;    // fall through
    case 3: a += (uint32_t)k[2] << 16;    // fall through
    case 2: a += (uint32_t)k[1] << 8;     // fall through
    case 1: a += k[0]; break;
    case 0: return c;
  }
  c ^= b; c -= rot32(b, 14);
  a ^= c; a -= rot32(c, 11);
  b ^= a; b -= rot32(a, 25);
  c ^= b; c -= rot32(b, 16);
  a ^= c; a -= rot32(c, 4);
  b ^= a; b -= rot32(a, 14);
  c ^= b; c -= rot32(b, 24);
  return c;
}

// ---- file builder -------------------------------------------------------
constexpr uint64_t kUndef = ~0ull;

struct Bytes {
  std::vector<uint8_t> v;
  void u8(uint8_t x) { v.push_back(x); }
  void u16(uint16_t x) { for (int i = 0; i < 2; i++) v.push_back((uint8_t)(x >> (8 * i))); }
  void u32(uint32_t x) { for (int i = 0; i < 4; i++) v.push_back((uint8_t)(x >> (8 * i))); }
  void u64(uint64_t x) { for (int i = 0; i < 8; i++) v.push_back((uint8_t)(x >> (8 * i))); }
  void raw(const void *p, size_t n) {
    const uint8_t *b = (const uint8_t *)p;
    v.insert(v.end(), b, b + n);
  }
};

// element types of datasets and attributes
enum class H5T { F64, U32, U8, STR };

struct Attr {
  std::string name;
  H5T t;
  std::vector<uint8_t> data;  // little-endian values
  size_t count = 1;           // elements
  bool scalar = true;         // rank 0 (else rank 1 of count)
  size_t strsize = 0;         // fixed string size (STR)
};

static void put_datatype(Bytes &m, H5T t, size_t strsize) {
  switch (t) {
    case H5T::F64:  // class 1 (floating point), version 1, IEEE 754 binary64 little-endian
      m.u8(0x11);
      m.u8(0x20);  // mantissa normalisation: implied leading 1
      m.u8(63);    // sign bit position
      m.u8(0);
      m.u32(8);
      m.u16(0);    // bit offset
      m.u16(64);   // precision
      m.u8(52);    // exponent location
      m.u8(11);    // exponent size
      m.u8(0);     // mantissa location
      m.u8(52);    // mantissa size
      m.u32(1023); // exponent bias
      break;
    case H5T::U32:  // class 0 (fixed point), unsigned little-endian
    case H5T::U8:
      m.u8(0x10);
      m.u8(0);
      m.u8(0);
      m.u8(0);
      m.u32(t == H5T::U32 ? 4 : 1);
      m.u16(0);
      m.u16(t == H5T::U32 ? 32 : 8);
      break;
    case H5T::STR:  // class 3 (string), null-terminated ASCII of fixed size
      m.u8(0x13);
      m.u8(0);
      m.u8(0);
      m.u8(0);
      m.u32((uint32_t)strsize);
      break;
  }
}

static void put_dataspace(Bytes &m, const std::vector<uint64_t> &dims, bool scalar) {
  m.u8(2);  // version 2
  m.u8(scalar ? 0 : (uint8_t)dims.size());
  m.u8(0);  // no maximum dimensions
  m.u8(scalar ? 0 : 1);  // scalar / simple
  if (!scalar)
    for (uint64_t d : dims) m.u64(d);
}

// object header message: type, body
struct Msg {
  uint8_t type;
  Bytes body;
};

static Msg attr_msg(const Attr &a) {
  Msg m;
  m.type = 0x0C;
  Bytes dt, ds;
  put_datatype(dt, a.t, a.strsize);
  put_dataspace(ds, {(uint64_t)a.count}, a.scalar);
  m.body.u8(3);  // version 3
  m.body.u8(0);
  m.body.u16((uint16_t)(a.name.size() + 1));
  m.body.u16((uint16_t)dt.v.size());
  m.body.u16((uint16_t)ds.v.size());
  m.body.u8(0);  // ASCII name
  m.body.raw(a.name.c_str(), a.name.size() + 1);
  m.body.raw(dt.v.data(), dt.v.size());
  m.body.raw(ds.v.data(), ds.v.size());
  m.body.raw(a.data.data(), a.data.size());
  return m;
}

class H5File {
 public:
  // raw data block; returns its file address
  uint64_t put_raw(const void *p, size_t n) {
    const uint64_t at = kBase + f_.v.size();
    f_.raw(p, n);
    return at;
  }
  // version 2 object header of the messages; returns its address
  uint64_t put_header(const std::vector<Msg> &msgs) {
    Bytes h;
    h.raw("OHDR", 4);
    h.u8(2);     // version
    h.u8(0x02);  // chunk 0 size in 4 bytes; no times, no attribute phase change
    size_t sz = 0;
    for (auto &m : msgs) sz += 4 + m.body.v.size();
    h.u32((uint32_t)sz);
    for (auto &m : msgs) {
      h.u8(m.type);
      h.u16((uint16_t)m.body.v.size());
      h.u8(0);  // message flags
      h.raw(m.body.v.data(), m.body.v.size());
    }
    h.u32(lookup3(h.v.data(), h.v.size(), 0));
    return put_raw(h.v.data(), h.v.size());
  }
  std::vector<uint8_t> finish(uint64_t root) {
    Bytes sb;
    sb.raw("\x89HDF\r\n\x1a\n", 8);
    sb.u8(2);  // superblock version 2
    sb.u8(8);  // size of offsets
    sb.u8(8);  // size of lengths
    sb.u8(0);  // file consistency flags
    sb.u64(0);                    // base address
    sb.u64(kUndef);               // superblock extension
    sb.u64(kBase + f_.v.size());  // end of file
    sb.u64(root);                 // root group object header
    sb.u32(lookup3(sb.v.data(), sb.v.size(), 0));
    std::vector<uint8_t> out = sb.v;
    out.insert(out.end(), f_.v.begin(), f_.v.end());
    return out;
  }

 private:
  static constexpr uint64_t kBase = 48;  // the superblock's size
  Bytes f_;
};

// ---- the openPMD tree ---------------------------------------------------
struct Node {
  std::string name;
  std::vector<Attr> attrs;
  std::vector<Node> kids;
  bool dataset = false;
  std::vector<uint64_t> dims;
  std::vector<uint8_t> data;  // FP64 values
  Node &kid(const std::string &n) {
    for (auto &k : kids)
      if (k.name == n) return k;
    kids.push_back(Node{});
    kids.back().name = n;
    return kids.back();
  }
};

static Attr a_str(const std::string &n, const std::string &s) {
  Attr a;
  a.name = n;
  a.t = H5T::STR;
  a.strsize = s.size() + 1;
  a.data.assign(s.begin(), s.end());
  a.data.push_back(0);
  return a;
}
static Attr a_f64(const std::string &n, const std::vector<double> &v, bool scalar = false) {
  Attr a;
  a.name = n;
  a.t = H5T::F64;
  a.count = v.size();
  a.scalar = scalar && v.size() == 1;
  a.data.resize(8 * v.size());
  std::memcpy(a.data.data(), v.data(), a.data.size());
  return a;
}
static Attr a_u32(const std::string &n, uint32_t v) {
  Attr a;
  a.name = n;
  a.t = H5T::U32;
  a.data.resize(4);
  std::memcpy(a.data.data(), &v, 4);
  return a;
}
static Attr a_u8(const std::string &n, uint8_t v) {
  Attr a;
  a.name = n;
  a.t = H5T::U8;
  a.data = {v};
  return a;
}

static uint64_t write_node(H5File &F, const Node &n) {
  std::vector<std::pair<std::string, uint64_t>> links;
  for (auto &k : n.kids) links.emplace_back(k.name, write_node(F, k));
  std::vector<Msg> msgs;
  if (n.dataset) {
    const uint64_t at = F.put_raw(n.data.data(), n.data.size());
    Msg ds;
    ds.type = 0x01;
    put_dataspace(ds.body, n.dims, false);
    msgs.push_back(std::move(ds));
    Msg dt;
    dt.type = 0x03;
    put_datatype(dt.body, H5T::F64, 0);
    msgs.push_back(std::move(dt));
    Msg fv;  // fill value, version 3: allocation early, written if set, none defined
    fv.type = 0x05;
    fv.body.u8(3);
    fv.body.u8(0x09);
    msgs.push_back(std::move(fv));
    Msg ly;  // data layout, version 3, contiguous
    ly.type = 0x08;
    ly.body.u8(3);
    ly.body.u8(1);
    ly.body.u64(at);
    ly.body.u64(n.data.size());
    msgs.push_back(std::move(ly));
  } else {
    Msg li;  // link info, version 0: no creation order, compact storage
    li.type = 0x02;
    li.body.u8(0);
    li.body.u8(0);
    li.body.u64(kUndef);
    li.body.u64(kUndef);
    msgs.push_back(std::move(li));
    Msg gi;  // group info, version 0
    gi.type = 0x0A;
    gi.body.u8(0);
    gi.body.u8(0);
    msgs.push_back(std::move(gi));
    for (auto &l : links) {
      Msg lk;  // link, version 1: hard link, 1-byte name length
      lk.type = 0x06;
      lk.body.u8(1);
      lk.body.u8(0);
      lk.body.u8((uint8_t)l.first.size());
      lk.body.raw(l.first.data(), l.first.size());
      lk.body.u64(l.second);
      msgs.push_back(std::move(lk));
    }
  }
  for (auto &a : n.attrs) msgs.push_back(attr_msg(a));
  return F.put_header(msgs);
}

static Node dataset_f64(const std::string &name, const std::vector<uint64_t> &dims, const double *p, size_t n) {
  Node d;
  d.name = name;
  d.dataset = true;
  d.dims = dims;
  d.data.resize(8 * n);
  if (n) std::memcpy(d.data.data(), p, 8 * n);
  return d;
}

// unitDimension (L, M, T, I, θ, N, J) of openpmd/root.jl's usi
static std::vector<double> dims7(double L, double M, double T, double I) { return {L, M, T, I, 0, 0, 0}; }

static void field_attrs(Node &n, const Ctx *c, const std::vector<double> &ud, bool comp) {
  n.attrs.push_back(a_f64("unitDimension", ud));
  n.attrs.push_back(a_f64("timeOffset", {0.0}, true));
  n.attrs.push_back(a_str("axisLabels", "xy"));
  n.attrs.push_back(a_str("dataOrder", "C"));
  n.attrs.push_back(a_str("geometry", "cartesian"));
  n.attrs.push_back(a_str("geometryParameters", ""));
  n.attrs.push_back(a_f64("gridGlobalOffset", {0.0, 0.0}));
  n.attrs.push_back(a_f64("gridSpacing", {c->g.dx, c->g.dy}));
  n.attrs.push_back(a_f64("gridUnitSI", {1.0}, true));
  n.attrs.push_back(a_str("fieldSmoothing", "none"));
  auto leaf = [&](Node &d) {
    d.attrs.push_back(a_f64("position", {0.0, 0.0}));
    d.attrs.push_back(a_f64("unitSI", {1.0}, true));
  };
  if (comp)
    for (auto &k : n.kids) leaf(k);
  else
    leaf(n);
}

// particle record metadata (openpmd/particles.jl ParticleRecordMetadata)
static void particle_attrs(Node &r, const std::vector<double> &ud, bool weighted) {
  r.attrs.push_back(a_f64("unitDimension", ud));
  r.attrs.push_back(a_f64("timeOffset", {0.0}, true));
  r.attrs.push_back(a_u8("macroWeighted", weighted ? 1 : 0));
  r.attrs.push_back(a_f64("weightingPower", {1.0}, true));
}

}  // namespace iskra

using namespace iskra;

extern "C" int iskra_write_openpmd(iskra_ctx *h, const char *prefix, int64_t iteration, double time, double dt,
                                   const char *const *species_names, int particles) {
  if (!h || !prefix) return ISKRA_EINVAL;
  Ctx *c = &h->c;
  const int nx = c->nx, ny = c->ny, nn = c->nn, ns = (int)c->species.size();
  const std::vector<uint64_t> fdims = {(uint64_t)ny, (uint64_t)nx};  // x fastest (Julia order)
  auto name_of = [&](int s) {
    return (species_names && species_names[s]) ? std::string(species_names[s]) : "s" + std::to_string(s);
  };
  Node root;
  // openpmd/root.jl RootMetadata
  root.attrs.push_back(a_str("openPMD", "1.1.0"));
  root.attrs.push_back(a_u32("openPMDextension", 1));
  root.attrs.push_back(a_str("iterationEncoding", "fileBased"));
  root.attrs.push_back(a_str("iterationFormat", "data%T.h5"));
  root.attrs.push_back(a_str("basePath", "/data/%T"));
  root.attrs.push_back(a_str("meshesPath", "fields/"));
  root.attrs.push_back(a_str("particlesPath", "particles/"));
  root.attrs.push_back(a_str("software", "iskra"));
  root.attrs.push_back(a_str("softwareVersion", "iskra_gb300"));
  {
    char buf[32];
    const std::time_t now = std::time(nullptr);
    std::strftime(buf, sizeof buf, "%Y/%m/%d %H:%M", std::localtime(&now));
    root.attrs.push_back(a_str("date", buf));
  }
  Node &it = root.kid("data").kid(std::to_string((long long)iteration));
  it.attrs.push_back(a_f64("dt", {dt}, true));
  it.attrs.push_back(a_f64("time", {time}, true));
  it.attrs.push_back(a_f64("timeUnitSI", {1.0}, true));
  Node &fields = it.kid("fields");
  // openpmd/fields.jl FieldMetadata
  fields.attrs.push_back(a_str("fieldSolver", "other"));
  fields.attrs.push_back(a_str("fieldSolverParameters", "Nagel"));
  fields.attrs.push_back(a_str("currentSmoothing", "none"));
  fields.attrs.push_back(a_str("chargeCorrection", "none"));
  std::vector<double> buf((size_t)3 * nn);
  // ρ, ϕ, E (ParticleInCell.jl:130-132), densities (:123)
  int rc = iskra_field_download(h, ISKRA_FIELD_RHO, buf.data());
  if (rc) return rc;
  fields.kids.push_back(dataset_f64("rho", fdims, buf.data(), nn));
  field_attrs(fields.kids.back(), c, dims7(-3, 0, 1, 1), false);
  if (c->ps) {
    rc = iskra_field_download(h, ISKRA_FIELD_PHI, buf.data());
    if (rc) return rc;
    fields.kids.push_back(dataset_f64("phi", fdims, buf.data(), nn));
    field_attrs(fields.kids.back(), c, dims7(2, 1, -3, -1), false);
  }
  rc = iskra_field_download(h, ISKRA_FIELD_E, buf.data());
  if (rc) return rc;
  {
    Node &E = fields.kid("E");
    E.kids.push_back(dataset_f64("x", fdims, buf.data(), nn));
    E.kids.push_back(dataset_f64("y", fdims, buf.data() + nn, nn));
    E.kids.push_back(dataset_f64("z", fdims, buf.data() + 2 * (size_t)nn, nn));
    field_attrs(E, c, dims7(1, 1, -3, -1), true);
  }
  for (int s = 0; s < ns; s++) {
    rc = iskra_density(h, s, buf.data());
    if (rc) return rc;
    fields.kids.push_back(dataset_f64("n" + name_of(s), fdims, buf.data(), nn));
    field_attrs(fields.kids.back(), c, dims7(-2, 0, 0, 0), false);
  }
  // accepted MCC collisions per node and process (mcc.jl:287)
  for (int m = 0; m < (int)c->mccs.size(); m++) {
    const int np_ = mcc_nproc(c, m);
    std::vector<unsigned> nu((size_t)nn * np_);
    rc = mcc_download_nu(c, m, nu.data());
    if (rc) return rc;
    for (int k = 0; k < np_; k++) {
      for (int q = 0; q < nn; q++) buf[q] = (double)nu[(size_t)q * np_ + k];
      fields.kids.push_back(dataset_f64("nuMCC-" + name_of(mcc_src(c, m)) + "-" + std::to_string(k + 1), fdims,
                                        buf.data(), nn));
      field_attrs(fields.kids.back(), c, dims7(-2, 0, 0, 0), false);
    }
  }
  // circuit probes: charge, current, source voltage, device voltage
  if (c->cir_d) {
    double st[5];
    rc = iskra_circuit_state(h, st);
    if (rc) return rc;
    const CircuitDev &cd = c->cir_h;
    const double vsrc = cd.amp * std::sin(2 * M_PI * cd.freq * st[0]) + cd.dc;
    const struct {
      const char *n;
      double v;
      std::vector<double> ud;
    } probes[] = {{"Q1", st[2], dims7(0, 0, 1, 1)},
                  {"I1", st[1], dims7(0, 0, 0, 1)},
                  {"V1", vsrc, dims7(2, 1, -3, -1)},
                  {"Vext", st[4], dims7(2, 1, -3, -1)}};
    for (auto &p : probes) {
      fields.kids.push_back(dataset_f64(p.n, {1}, &p.v, 1));
      fields.kids.back().attrs.push_back(a_f64("unitDimension", p.ud));
      fields.kids.back().attrs.push_back(a_f64("unitSI", {1.0}, true));
    }
  }
  // particle records (ParticleInCell.jl:63-71)
  if (particles) {
    Node &parts = it.kid("particles");
    parts.attrs.push_back(a_f64("particleShape", {0.0}, true));
    parts.attrs.push_back(a_str("currentDeposition", "none"));
    parts.attrs.push_back(a_str("particlePush", "Boris"));
    parts.attrs.push_back(a_str("particleInterpolation", "other"));
    parts.attrs.push_back(a_str("particleSmoothing", "none"));
    for (int s = 0; s < ns; s++) {
      int64_t np = 0;
      rc = iskra_species_count(h, s, &np);
      if (rc) return rc;
      const int64_t ld = std::max<int64_t>(np, 1);
      std::vector<double> x((size_t)ld * 2), v((size_t)ld * 3);
      std::vector<uint32_t> id(ld);
      int64_t got = 0;
      rc = iskra_species_download(h, s, x.data(), v.data(), nullptr, id.data(), ld, &got);
      if (rc) return rc;
      const Species &sp = c->species[s];
      const uint64_t n = (uint64_t)got;
      Node &P = parts.kid(name_of(s));
      Node &pos = P.kid("position");
      pos.kids.push_back(dataset_f64("x", {n}, x.data(), n));
      pos.kids.push_back(dataset_f64("y", {n}, x.data() + ld, n));
      for (auto &k : pos.kids) k.attrs.push_back(a_f64("unitSI", {1.0}, true));
      particle_attrs(pos, dims7(1, 0, 0, 0), false);
      Node &mom = P.kid("momentum");
      std::vector<double> pm((size_t)3 * n);
      for (size_t k = 0; k < 3; k++)
        for (size_t q = 0; q < n; q++) pm[k * n + q] = sp.m * v[k * (size_t)ld + q];
      const char *cn[3] = {"x", "y", "z"};
      for (int k = 0; k < 3; k++) mom.kids.push_back(dataset_f64(cn[k], {n}, pm.data() + k * n, n));
      for (auto &k : mom.kids) k.attrs.push_back(a_f64("unitSI", {1.0}, true));
      particle_attrs(mom, dims7(1, 1, -1, 0), false);
      std::vector<double> wg(n, sp.w0), idd(id.begin(), id.begin() + n);
      P.kids.push_back(dataset_f64("weighting", {n}, wg.data(), n));
      P.kids.back().attrs.push_back(a_f64("unitSI", {1.0}, true));
      particle_attrs(P.kids.back(), dims7(0, 0, 0, 0), true);
      P.kids.push_back(dataset_f64("id", {n}, idd.data(), n));
      P.kids.back().attrs.push_back(a_f64("unitSI", {1.0}, true));
      particle_attrs(P.kids.back(), dims7(0, 0, 0, 0), false);
      // constant records (a value and a shape instead of a dataset)
      const struct {
        const char *n;
        double v;
        std::vector<double> ud;
      } cst[] = {{"charge", sp.q, dims7(0, 0, 1, 1)}, {"mass", sp.m, dims7(0, 1, 0, 0)}};
      for (auto &q : cst) {
        Node &r = P.kid(q.n);
        r.attrs.push_back(a_f64("value", {q.v}, true));
        r.attrs.push_back(a_f64("shape", {(double)n}));
        r.attrs.push_back(a_f64("unitSI", {1.0}, true));
        particle_attrs(r, q.ud, false);
      }
      Node &off = P.kid("positionOffset");
      for (const char *k : {"x", "y", "z"}) {
        Node &r = off.kid(k);
        r.attrs.push_back(a_f64("value", {0.0}, true));
        r.attrs.push_back(a_f64("shape", {(double)n}));
        r.attrs.push_back(a_f64("unitSI", {1.0}, true));
      }
      particle_attrs(off, dims7(1, 0, 0, 0), false);
    }
  }
  // <prefix>/hdf5/data<iteration>.h5 (hdf5.jl:50-52)
  H5File F;
  const uint64_t root_at = write_node(F, root);
  const std::vector<uint8_t> bytes = F.finish(root_at);
  const std::string dir = std::string(prefix) + "/hdf5";
  mkdir(prefix, 0755);
  mkdir(dir.c_str(), 0755);
  const std::string path = dir + "/data" + std::to_string((long long)iteration) + ".h5";
  FILE *f = std::fopen(path.c_str(), "wb");
  if (!f) return set_err(c, ISKRA_EINVAL, "cannot open " + path);
  const size_t wr = std::fwrite(bytes.data(), 1, bytes.size(), f);
  const int cl = std::fclose(f);
  if (wr != bytes.size() || cl != 0) return set_err(c, ISKRA_EINVAL, "short write to " + path);
  return ISKRA_OK;
}
