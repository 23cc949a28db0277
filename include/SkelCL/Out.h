// Tag for a container a skeleton writes (include/SkelCL/Out.h:65-97).
#ifndef SKELCL_OUT_H_
#define SKELCL_OUT_H_

namespace skelcl {

template <typename> class Out;

template <template <typename> class ContainerType, typename T>
class Out<ContainerType<T>> {
public:
  Out(ContainerType<T>& c) : _container(c) {}
  ContainerType<T>& container() const { return _container; }

private:
  ContainerType<T>& _container;
};

template <template <typename> class ContainerType, typename T>
Out<ContainerType<T>> out(ContainerType<T>& c) {
  return Out<ContainerType<T>>(c);
}

}  // namespace skelcl

#endif  // SKELCL_OUT_H_
