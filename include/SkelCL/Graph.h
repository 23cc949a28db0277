// skelcl::Graph: a sequence of skeleton calls captured once and replayed with
// one launch (CUDA graphs; no counterpart in the reference).
//
//   skelcl::Graph g;
//   g.capture([&] { zip(out(z), x, y); reduce(out(r), z); });
//   for (...) g.launch();            // same containers, new contents
//
// capture() runs the body once normally (uploading inputs, sizing workspaces
// and compiling lazily built variants), then records it.  Inside the body use
// containers that already live on the device and Out<> outputs of the right
// size: host transfers cannot be recorded.  Between replays, new input
// contents go to the device as usual (dataOnHostModified(), then
// copyDataToDevices()), and outputs read on the host after launch() need
// dataOnDeviceModified() first: a replay runs on the device only.
#ifndef SKELCL_GRAPH_H_
#define SKELCL_GRAPH_H_

#include <pvsutil/Assert.h>

#include "detail/Runtime.h"

namespace skelcl {

class Graph {
public:
  Graph() = default;
  Graph(const Graph&) = delete;
  Graph& operator=(const Graph&) = delete;
  ~Graph() {
    if (_g && scl_is_initialized()) scl_graph_destroy(_g);
  }

  template <typename F>
  void capture(F body) {
    body();
    detail::checkStatus(scl_sync(), "Graph warm-up");
    if (_g) {
      scl_graph_destroy(_g);
      _g = nullptr;
    }
    detail::checkStatus(scl_graph_begin(), "Graph capture");
    body();
    detail::checkStatus(scl_graph_end(&_g), "Graph capture");
  }
  void launch() const {
    ASSERT_MESSAGE(_g != nullptr, "Graph::launch before capture");
    detail::checkStatus(scl_graph_launch(_g), "Graph launch");
  }
  // waits for everything launched so far
  static void wait() { detail::checkStatus(scl_sync(), "Graph wait"); }

private:
  scl_graph* _g = nullptr;
};

// Autotuning of launch shapes (block size, items per thread, tile shapes):
// off unless SKELCL_AUTOTUNE=1 or switched on here.
inline void setAutotune(bool on) { detail::checkStatus(scl_autotune_set(on ? 1 : 0), "setAutotune"); }

}  // namespace skelcl

#endif  // SKELCL_GRAPH_H_
