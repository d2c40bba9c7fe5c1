// Instance-fold analysis (see instance_fold.h).
#include "instance_fold.h"

#include <set>

namespace rrtl {

namespace {

std::string quote(const std::string& s) {
  std::string o = "\"";
  for (char c : s) {
    if (c == '"' || c == '\\') o += '\\';
    o += c;
  }
  return o + "\"";
}

const SignalInfo* port_of(const Module& m, const std::string& name) {
  for (const SignalInfo& s : m.signals)
    if (s.name == name && (s.kind == SigKind::Input || s.kind == SigKind::Output || s.kind == SigKind::Inout)) return &s;
  return nullptr;
}

}  // namespace

std::optional<InstanceFold> analyze_instance_fold(const Design& d, const std::string& top, std::string* why) {
  auto no = [&](const std::string& w) -> std::optional<InstanceFold> {
    if (why) *why = w;
    return std::nullopt;
  };
  const Module* m = d.find_module(top);
  if (!m) return no("no module `" + top + "`");
  if (m->instances.size() < 2) return no("`" + top + "` has fewer than two instances");
  for (const SignalInfo& s : m->signals)
    if (s.kind == SigKind::Reg || s.kind == SigKind::Mem) return no("`" + top + "` has registers or memories of its own");
  if (!m->assignments.empty() || !m->memory_writes.empty()) return no("`" + top + "` has logic of its own");
  const std::string& child = m->instances[0].module;
  for (const Instance& in : m->instances)
    if (in.module != child) return no("the instances are of different modules");
  const Module* c = d.find_module(child);
  if (!c) return no("no module `" + child + "`");
  if (c->is_external) return no("`" + child + "` is external");

  InstanceFold f;
  f.child = child;
  std::set<uint32_t> ins, outs;
  for (uint32_t i = 0; i < m->instances.size(); ++i) {
    const Instance& in = m->instances[i];
    f.instance_names.push_back(in.name);
    for (const auto& conn : in.connections) {
      const SignalInfo* p = port_of(*c, conn.first);
      if (!p) return no("`" + child + "` has no port `" + conn.first + "`");
      if (p->kind == SigKind::Inout) return no("inout port `" + conn.first + "` is not folded");
      const SignalInfo* ts = m->signal(conn.second);
      if (!ts) return no("instance `" + in.name + "` connects to a signal outside `" + top + "`");
      const bool out = p->kind == SigKind::Output;
      if (out) {
        if (!outs.insert(conn.second.id).second) return no("two instance outputs drive `" + ts->name + "`");
      } else {
        ins.insert(conn.second.id);
      }
      f.connections.push_back(FoldConnection{ts->name, i, conn.first, out});
    }
  }
  for (uint32_t s : outs)
    if (ins.count(s)) return no("an instance output feeds an instance input");
  return f;
}

std::string instance_fold_json(const InstanceFold& f) {
  std::string o = "{\"child\": " + quote(f.child) + ", \"instances\": [";
  for (size_t i = 0; i < f.instance_names.size(); ++i) o += (i ? ", " : "") + quote(f.instance_names[i]);
  o += "], \"connections\": [";
  for (size_t i = 0; i < f.connections.size(); ++i) {
    const FoldConnection& c = f.connections[i];
    o += (i ? ", [" : "[") + quote(c.top_signal) + ", " + std::to_string(c.instance) + ", " + quote(c.port) + ", " +
         (c.output ? "\"out\"" : "\"in\"") + "]";
  }
  return o + "]}";
}

}  // namespace rrtl
