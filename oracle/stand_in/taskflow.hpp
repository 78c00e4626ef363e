// Stand-in for the taskflow header the reference includes as "taskflow.hpp"
// (taskflow/taskflow). Only contraction variants outside fastcc_multiply use
// it; tasks run one after another on the calling thread.
#pragma once
#include <cstddef>
#include <functional>
#include <vector>

namespace tf {
class Taskflow {
 public:
  template <class F> void emplace(F &&f) { tasks.emplace_back(std::forward<F>(f)); }
  std::vector<std::function<void()>> tasks;
};
class Executor {
 public:
  explicit Executor(std::size_t = 0) {}
  int this_worker_id() const { return 0; }
  struct Done { void wait() {} };
  Done run(Taskflow &t) {
    for (auto &f : t.tasks) f();
    return {};
  }
};
}  // namespace tf
