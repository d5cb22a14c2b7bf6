// Zero-copy export of a vta_device_array as a DLPack managed tensor
// (vta_device_array_to_dlpack), the C side of the crate's
// DeviceArrayF32Py::__dlpack__ (src/utilities/dlpack_cuda.rs:265-374): the
// array's device buffer moves into the managed tensor, whose deleter frees it
// on the array's device.  The Python binding wraps the result in a
// "dltensor" / "dltensor_versioned" capsule.
//
// The structs follow the public DLPack ABI (dlpack.h v0.8 / v1.x): DLTensor,
// DLManagedTensor and DLManagedTensorVersioned must have exactly this layout
// for a consumer (torch, cupy, jax) to read them.
#include <cstdint>
#include <cstdlib>

#include "vta_internal.h"

namespace {

struct DLDevice {
    int32_t device_type;  // kDLCUDA = 2
    int32_t device_id;
};
struct DLDataType {
    uint8_t code;  // kDLFloat = 2
    uint8_t bits;
    uint16_t lanes;
};
struct DLTensor {
    void* data;
    DLDevice device;
    int32_t ndim;
    DLDataType dtype;
    int64_t* shape;
    int64_t* strides;  // in elements
    uint64_t byte_offset;
};
struct DLManagedTensor {
    DLTensor dl_tensor;
    void* manager_ctx;
    void (*deleter)(DLManagedTensor*);
};
struct DLPackVersion {
    uint32_t major, minor;
};
struct DLManagedTensorVersioned {
    DLPackVersion version;
    void* manager_ctx;
    void (*deleter)(DLManagedTensorVersioned*);
    uint64_t flags;
    DLTensor dl_tensor;
};

// Owns the exported buffer and the shape / strides the tensor points to.
struct Manager {
    void* data;
    int device;
    int64_t shape[2];
    int64_t strides[2];
};

void release(Manager* m) {
    if (!m) return;
    if (m->data) {
        int cur = 0;
        cudaGetDevice(&cur);
        cudaSetDevice(m->device);
        cudaFree(m->data);
        cudaSetDevice(cur);
    }
    std::free(m);
}

void delete_legacy(DLManagedTensor* t) {
    if (!t) return;
    release(static_cast<Manager*>(t->manager_ctx));
    std::free(t);
}

void delete_versioned(DLManagedTensorVersioned* t) {
    if (!t) return;
    release(static_cast<Manager*>(t->manager_ctx));
    std::free(t);
}

DLTensor tensor_of(Manager* m) {
    DLTensor d{};
    d.data = m->data;
    d.device = DLDevice{2, m->device};
    d.ndim = 2;
    d.dtype = DLDataType{2, 32, 1};
    d.shape = m->shape;
    d.strides = m->strides;
    d.byte_offset = 0;
    return d;
}

}  // namespace

using namespace vta;

extern "C" {

vta_status vta_device_array_to_dlpack(vta_device_array* arr, int versioned, void** out_managed) {
    if (!arr || !out_managed) return fail(VTA_ERR_INVALID_INPUT, "dlpack: null argument");
    *out_managed = nullptr;
    auto* m = static_cast<Manager*>(std::malloc(sizeof(Manager)));
    if (!m) return fail(VTA_ERR_OUT_OF_MEMORY, "dlpack: host allocation failed");
    m->data = arr->ptr;
    m->device = arr->device;
    m->shape[0] = (int64_t)arr->rows;
    m->shape[1] = (int64_t)arr->cols;
    m->strides[0] = (int64_t)arr->cols;
    m->strides[1] = 1;
    if (versioned) {
        auto* t = static_cast<DLManagedTensorVersioned*>(std::malloc(sizeof(DLManagedTensorVersioned)));
        if (!t) {
            std::free(m);
            return fail(VTA_ERR_OUT_OF_MEMORY, "dlpack: host allocation failed");
        }
        t->version = DLPackVersion{1, 0};
        t->manager_ctx = m;
        t->deleter = delete_versioned;
        t->flags = 0;
        t->dl_tensor = tensor_of(m);
        *out_managed = t;
    } else {
        auto* t = static_cast<DLManagedTensor*>(std::malloc(sizeof(DLManagedTensor)));
        if (!t) {
            std::free(m);
            return fail(VTA_ERR_OUT_OF_MEMORY, "dlpack: host allocation failed");
        }
        t->dl_tensor = tensor_of(m);
        t->manager_ctx = m;
        t->deleter = delete_legacy;
        *out_managed = t;
    }
    // the buffer now belongs to the managed tensor
    arr->ptr = nullptr;
    arr->rows = arr->cols = 0;
    return VTA_OK;
}

vta_status vta_dlpack_delete(void* managed, int versioned) {
    if (!managed) return VTA_OK;
    if (versioned) {
        auto* t = static_cast<DLManagedTensorVersioned*>(managed);
        if (t->deleter) t->deleter(t);
    } else {
        auto* t = static_cast<DLManagedTensor*>(managed);
        if (t->deleter) t->deleter(t);
    }
    return VTA_OK;
}

}  // extern "C"
