// Stand-in for onika's operator node API: OperatorNode, ADD_SLOT slots with
// their access (*slot, slot->, has_value()), fatal_error(), the execution
// context's GPU stream and onika::data_file_path.
#pragma once
#include <cstddef>
#include <cstdint>
#include <memory>
#include <optional>
#include <ostream>
#include <string>
#include <sys/types.h>

namespace onika {
namespace scg {
struct DocString {
  std::string text;
};
enum SlotDir { INPUT, OUTPUT, INPUT_OUTPUT, PRIVATE };
struct RequiredTag {};
struct OptionalTag {};
constexpr RequiredTag REQUIRED{};
constexpr OptionalTag OPTIONAL{};

template <class T>
class OperatorSlot {
 public:
  OperatorSlot(SlotDir = INPUT) {}
  OperatorSlot(SlotDir, RequiredTag, DocString = {}) {}
  OperatorSlot(SlotDir, OptionalTag, DocString = {}) : m_set(false) {}
  template <class V>
  OperatorSlot(SlotDir, const V& v, DocString = {}) : m_value(v) {}
  T& operator*() { return m_value; }
  const T& operator*() const { return m_value; }
  T* operator->() { return &m_value; }
  const T* operator->() const { return &m_value; }
  bool has_value() const { return m_set; }

 private:
  T m_value{};
  bool m_set = true;
};

class OperatorNode {
 public:
  virtual ~OperatorNode() = default;
  virtual void execute() = 0;
};

struct FatalStream {
  std::ostream& os;
  template <class T>
  FatalStream& operator<<(const T& v) {
    os << v;
    return *this;
  }
  FatalStream& operator<<(std::ostream& (*m)(std::ostream&)) {
    os << m;
    return *this;
  }
};
FatalStream fatal_error();

struct ParallelExecutionContext {
  void* gpu_stream() const { return nullptr; }
};
ParallelExecutionContext* parallel_execution_context();
}  // namespace scg

std::string data_file_path(const std::string& f);
}  // namespace onika

#define ADD_SLOT(T, name, ...) ::onika::scg::OperatorSlot<T> name{__VA_ARGS__}

namespace exanb {
using namespace ::onika::scg;
}
