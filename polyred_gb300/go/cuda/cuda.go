// Package cuda binds libpolyred_cuda.so (include/polyred_cuda.h) for the Go
// renderer through purego, keeping polyred cgo-free. It is the Go half of the
// render.CUDA(dev) option; see INTEGRATION.md for the render package hook.
//
// The library is opened like the reference opens its graphics drivers
// (gpu/backend_gl_lib_linux.go:18-25): purego.Dlopen + RegisterLibFunc. Every
// entry point takes integers and pointers only.
package cuda

import (
	"errors"
	"fmt"
	"os"
	"runtime"
	"sync"
	"unsafe"

	"github.com/ebitengine/purego"
)

// Status codes (PR_* in include/polyred_cuda.h).
const (
	OK             = 0
	ErrInvalidArg  = -1
	ErrOOM         = -2
	ErrCUDA        = -3
	ErrOverflow    = -4
	ErrTimeout     = -5
	ErrUnimpl      = -6
	ErrNoScene     = -7
	ErrUnsupported = -8
	ErrNoDevice    = -9
	ErrSingular    = -10
)

const (
	MatFlatShading   = 1
	MatAO            = 2
	MatReceiveShadow = 4
	MatMipmap        = 8

	LightPoint       = 0
	LightDirectional = 1

	FramePerspective = 1
	FrameShadowMap   = 2
	FrameGamma       = 4

	TriNone = 0xFFFFFFFF
)

// Object mirrors pr_object.
type Object struct {
	FirstTri uint32
	NTris    uint32
	MatBase  int32
	_        uint32
	Model    [16]float32
}

// Material mirrors pr_material.
type Material struct {
	Diffuse     [4]uint8
	Specular    [4]uint8
	Texture     [4]uint8
	Shininess   float32
	Flags       uint32
	TextureSize int32
}

// SceneDesc mirrors pr_scene_desc.
type SceneDesc struct {
	Size       uint32
	Flags      uint32
	NTris      uint32
	NObjects   uint32
	NMaterials uint32
	_          uint32
	Pos        *float32
	Nor        *float32
	UV         *float32
	Col        *uint8
	MatID      *int32
	Objects    *Object
	Materials  *Material
	// Textures is nil or one entry per material: the image of a
	// buffer.NewTexture(TextureImage(img)) (RGBA nil keeps the uniform texel).
	Textures *Texture
}

// Texture mirrors pr_texture: an *image.RGBA's size and Pix (rows top-down).
type Texture struct {
	Width, Height int32
	RGBA          *uint8
}

// Light mirrors pr_light.
type Light struct {
	Type       int32
	CastShadow int32
	Pos        [3]float32
	Dir        [3]float32
	Intensity  float32
	Color      [4]uint8
	ShadowView [16]float32
	ShadowProj [16]float32
}

// FrameDesc mirrors pr_frame_desc.
type FrameDesc struct {
	Size         uint32
	Flags        uint32
	Width        int32
	Height       int32
	View         [16]float32
	Proj         [16]float32
	CamPos       [3]float32
	Background   [4]uint8
	NLights      uint32
	NAmbient     uint32
	Lights       *Light
	Ambient      *float32
	ShadowWidth  int32
	ShadowHeight int32
	// MSAA is render.MSAA (0 or 1: none). With n > 1 the frame renders at
	// n*Width x n*Height and Outputs.RGBA receives the Width x Height image
	// after imageutil.Resize; the other outputs are framebuffer-sized.
	MSAA     int32
	Reserved int32
}

// Outputs mirrors pr_outputs; nil fields are not produced.
type Outputs struct {
	Size       uint32
	Flags      uint32
	RGBA       *uint8
	TriID      *uint32
	Depth      *float32
	Nor        *float32
	FaceNor    *float32
	WorldPos   *float32
	UVD        *float32
	VCol       *uint8
	MatID      *int32
	ShadowMaps *float32
}

var (
	loadOnce sync.Once
	loadErr  error

	prCreate       func(device int32, out *uintptr) int32
	prDestroy      func(ctx uintptr) int32
	prSceneUpload  func(ctx uintptr, s *SceneDesc) int32
	prShadowReset  func(ctx uintptr) int32
	prRender       func(ctx uintptr, f *FrameDesc, o *Outputs) int32
	prLastError    func() string
	prViewMatrix   func(pos, target, up *float32, out *float32) int32
	prShadowCamera func(lightPos, center, view, proj, outView, outProj *float32) int32
	prFrameSubmit  func(ctx uintptr, s *SceneDesc, f *FrameDesc, o *Outputs) int32
	prSync         func(ctx uintptr) int32
	prHostAlloc    func(bytes uintptr, out *unsafe.Pointer) int32
	prHostFree     func(p unsafe.Pointer) int32
)

// LibraryPath is where Open looks for the library unless POLYRED_CUDA_LIB
// is set.
var LibraryPath = "libpolyred_cuda.so"

func load() error {
	loadOnce.Do(func() {
		path := LibraryPath
		if p := os.Getenv("POLYRED_CUDA_LIB"); p != "" {
			path = p
		}
		lib, err := purego.Dlopen(path, purego.RTLD_NOW|purego.RTLD_GLOBAL)
		if err != nil {
			loadErr = fmt.Errorf("cuda: %w", err)
			return
		}
		purego.RegisterLibFunc(&prCreate, lib, "pr_create")
		purego.RegisterLibFunc(&prDestroy, lib, "pr_destroy")
		purego.RegisterLibFunc(&prSceneUpload, lib, "pr_scene_upload")
		purego.RegisterLibFunc(&prShadowReset, lib, "pr_shadow_reset")
		purego.RegisterLibFunc(&prRender, lib, "pr_render")
		purego.RegisterLibFunc(&prLastError, lib, "pr_last_error")
		purego.RegisterLibFunc(&prViewMatrix, lib, "pr_view_matrix")
		purego.RegisterLibFunc(&prShadowCamera, lib, "pr_shadow_camera")
		purego.RegisterLibFunc(&prFrameSubmit, lib, "pr_frame_submit")
		purego.RegisterLibFunc(&prSync, lib, "pr_sync")
		purego.RegisterLibFunc(&prHostAlloc, lib, "pr_host_alloc")
		purego.RegisterLibFunc(&prHostFree, lib, "pr_host_free")
	})
	return loadErr
}

// Error is a non-OK status with the library's detail message.
type Error struct {
	Status int32
	Detail string
}

func (e *Error) Error() string { return fmt.Sprintf("cuda: %s (status %d)", e.Detail, e.Status) }

// ErrClosed is returned by a Device used after Close.
var ErrClosed = errors.New("cuda: device closed")

func check(st int32) error {
	if st == OK {
		return nil
	}
	return &Error{Status: st, Detail: prLastError()}
}

// Device is one render context on one GPU. The caller owns it: a renderer
// given a Device through render.CUDA never closes it.
type Device struct {
	mu  sync.Mutex
	ctx uintptr
}

// Open creates a context on CUDA device ordinal.
func Open(ordinal int) (*Device, error) {
	if err := load(); err != nil {
		return nil, err
	}
	var ctx uintptr
	if err := check(prCreate(int32(ordinal), &ctx)); err != nil {
		return nil, err
	}
	d := &Device{ctx: ctx}
	runtime.SetFinalizer(d, func(d *Device) { d.Close() })
	return d, nil
}

// Close releases the context and its device memory.
func (d *Device) Close() error {
	d.mu.Lock()
	defer d.mu.Unlock()
	if d.ctx == 0 {
		return nil
	}
	err := check(prDestroy(d.ctx))
	d.ctx = 0
	return err
}

// UploadScene copies a flattened scene to the device (and clears the shadow
// maps, as initShadowMaps does).
func (d *Device) UploadScene(s *SceneDesc) error {
	d.mu.Lock()
	defer d.mu.Unlock()
	if d.ctx == 0 {
		return ErrClosed
	}
	s.Size = uint32(unsafe.Sizeof(*s))
	err := check(prSceneUpload(d.ctx, s))
	runtime.KeepAlive(s)
	return err
}

// ResetShadows zeroes the persistent shadow maps.
func (d *Device) ResetShadows() error {
	d.mu.Lock()
	defer d.mu.Unlock()
	if d.ctx == 0 {
		return ErrClosed
	}
	return check(prShadowReset(d.ctx))
}

// Render runs shadows, forward raster, deferred shading and gamma for one
// frame and fills the requested outputs.
func (d *Device) Render(f *FrameDesc, o *Outputs) error {
	d.mu.Lock()
	defer d.mu.Unlock()
	if d.ctx == 0 {
		return ErrClosed
	}
	f.Size = uint32(unsafe.Sizeof(*f))
	o.Size = uint32(unsafe.Sizeof(*o))
	err := check(prRender(d.ctx, f, o))
	runtime.KeepAlive(f)
	runtime.KeepAlive(o)
	return err
}

// Submit uploads the scene and queues one frame without waiting
// (pr_frame_submit): the upload overlaps the frame before it, host outputs
// come back while the next frame computes. The scene's arrays and the
// outputs must stay valid and unchanged until Sync, so they should live
// outside the Go heap (HostAlloc) or be pinned by the caller.
func (d *Device) Submit(s *SceneDesc, f *FrameDesc, o *Outputs) error {
	d.mu.Lock()
	defer d.mu.Unlock()
	if d.ctx == 0 {
		return ErrClosed
	}
	s.Size = uint32(unsafe.Sizeof(*s))
	f.Size = uint32(unsafe.Sizeof(*f))
	o.Size = uint32(unsafe.Sizeof(*o))
	return check(prFrameSubmit(d.ctx, s, f, o))
}

// Sync waits for every submitted frame and its outputs.
func (d *Device) Sync() error {
	d.mu.Lock()
	defer d.mu.Unlock()
	if d.ctx == 0 {
		return ErrClosed
	}
	return check(prSync(d.ctx))
}

// ShadowCamera returns the light camera initShadowMaps fits around the main
// camera frustum (render/shadow.go:41-85), computed by the library with the
// reference's float32 evaluation order.
func ShadowCamera(lightPos, center [3]float32, view, proj [16]float32) (v, p [16]float32, err error) {
	if err = load(); err != nil {
		return
	}
	err = check(prShadowCamera(&lightPos[0], &center[0], &view[0], &proj[0], &v[0], &p[0]))
	return
}

// HostAlloc returns n bytes of page-locked host memory (pr_host_alloc) for
// frame outputs and scene arrays: the device copies to and from it at the
// link's full rate. The memory is outside the Go heap; free it with HostFree.
func HostAlloc(n uintptr) (unsafe.Pointer, error) {
	if err := load(); err != nil {
		return nil, err
	}
	var p unsafe.Pointer
	if err := check(prHostAlloc(n, &p)); err != nil {
		return nil, err
	}
	return p, nil
}

// HostFree releases memory from HostAlloc.
func HostFree(p unsafe.Pointer) error {
	if err := load(); err != nil {
		return err
	}
	return check(prHostFree(p))
}
