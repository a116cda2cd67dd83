// Package cuda binds libpolyred_cuda.so (include/polyred_cuda.h) for the Go
// renderer through purego, keeping polyred cgo-free. It is the Go half of the
// render.CUDA(dev) option.
//
// The library is opened like the reference opens its graphics drivers
// (gpu/backend_gl_lib_linux.go:18-25): purego.Dlopen + RegisterLibFunc. Every
// entry point takes integers and pointers only.
package cuda

import (
	"errors"
	"fmt"
	"image"
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
	ErrFatal       = -11
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
	prDeviceAlloc  func(ctx uintptr, bytes uintptr, out *unsafe.Pointer) int32
	prDeviceFree   func(ctx uintptr, p unsafe.Pointer) int32
	prDeviceRead   func(ctx uintptr, src unsafe.Pointer, bytes uintptr, dst unsafe.Pointer) int32
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
		purego.RegisterLibFunc(&prDeviceAlloc, lib, "pr_device_alloc")
		purego.RegisterLibFunc(&prDeviceFree, lib, "pr_device_free")
		purego.RegisterLibFunc(&prDeviceRead, lib, "pr_device_read")
		for _, f := range registerExtra {
			if err := f(lib); err != nil {
				loadErr = err
				return
			}
		}
	})
	return loadErr
}

// registerExtra binds the entry points of the binding's other files (diff.go).
var registerExtra []func(lib uintptr) error

// register binds C function name of lib to the Go function variable fptr.
func register(fptr any, lib uintptr, name string) error {
	sym, err := purego.Dlsym(lib, name)
	if err != nil {
		return fmt.Errorf("cuda: %s: %w", name, err)
	}
	purego.RegisterFunc(fptr, sym)
	return nil
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

// Fragment is one pixel of a GBuffer, the fields of buffer.Fragment
// (buffer/buffer.go) that the frame produces.
type Fragment struct {
	Ok         bool
	X, Y       int
	Depth      float32
	U, V       float32
	Du, Dv     float32
	Nor        [4]float32
	FaceNor    [4]float32
	WordPos    [4]float32
	Col        [4]uint8
	MaterialID int64
	TriID      uint32
}

// GBuffer is a frame's outputs kept in device memory: render into it with
// d.Render(f, g.Outputs()) and read the fragments or the image on demand,
// instead of copying every field of every pixel to the host after each pass
// (the per-pass marshal of render/gpudeferred.go:110-187). Fields are W x H
// (the framebuffer); rows are top-down, row r holding raster row H-1-r.
type GBuffer struct {
	dev    *Device
	W, H   int
	fields map[string]unsafe.Pointer
	out    Outputs
}

var gbufferFields = []struct {
	name  string
	bytes int
}{
	{"rgba", 4}, {"tri_id", 4}, {"depth", 4}, {"nor", 16}, {"face_nor", 16},
	{"world_pos", 16}, {"uvd", 16}, {"vcol", 4}, {"mat_id", 4},
}

// NewGBuffer allocates device outputs for w x h frames on d.
func (d *Device) NewGBuffer(w, h int) (*GBuffer, error) {
	if w <= 0 || h <= 0 {
		return nil, &Error{Status: -1, Detail: "GBuffer size must be positive"}
	}
	d.mu.Lock()
	ctx := d.ctx
	d.mu.Unlock()
	if ctx == 0 {
		return nil, ErrClosed
	}
	g := &GBuffer{dev: d, W: w, H: h, fields: map[string]unsafe.Pointer{}}
	for _, f := range gbufferFields {
		var p unsafe.Pointer
		if err := check(prDeviceAlloc(ctx, uintptr(w*h*f.bytes), &p)); err != nil {
			g.Free()
			return nil, err
		}
		g.fields[f.name] = p
	}
	g.out = Outputs{
		Flags:    1, // PR_OUT_DEVICE_PTRS
		RGBA:     (*uint8)(g.fields["rgba"]),
		TriID:    (*uint32)(g.fields["tri_id"]),
		Depth:    (*float32)(g.fields["depth"]),
		Nor:      (*float32)(g.fields["nor"]),
		FaceNor:  (*float32)(g.fields["face_nor"]),
		WorldPos: (*float32)(g.fields["world_pos"]),
		UVD:      (*float32)(g.fields["uvd"]),
		VCol:     (*uint8)(g.fields["vcol"]),
		MatID:    (*int32)(g.fields["mat_id"]),
	}
	runtime.SetFinalizer(g, func(g *GBuffer) { g.Free() })
	return g, nil
}

// Outputs is the pr_outputs that renders into this GBuffer.
func (g *GBuffer) Outputs() *Outputs { return &g.out }

func (g *GBuffer) read(name string, index, size int, dst unsafe.Pointer) error {
	src := unsafe.Add(g.fields[name], index*size)
	return check(prDeviceRead(g.dev.ctx, src, uintptr(size), dst))
}

// Fragment reads the fragment at raster (x, y) (FragmentBuffer.UnsafeGet).
func (g *GBuffer) Fragment(x, y int) (Fragment, error) {
	var f Fragment
	if x < 0 || y < 0 || x >= g.W || y >= g.H {
		return f, nil // FragmentBuffer.Get: the zero fragment outside the buffer
	}
	i := (g.H-1-y)*g.W + x
	var uvd [4]float32
	var mat int32
	reads := []struct {
		name string
		size int
		dst  unsafe.Pointer
	}{
		{"tri_id", 4, unsafe.Pointer(&f.TriID)}, {"depth", 4, unsafe.Pointer(&f.Depth)},
		{"nor", 16, unsafe.Pointer(&f.Nor)}, {"face_nor", 16, unsafe.Pointer(&f.FaceNor)},
		{"world_pos", 16, unsafe.Pointer(&f.WordPos)}, {"uvd", 16, unsafe.Pointer(&uvd)},
		{"vcol", 4, unsafe.Pointer(&f.Col)}, {"mat_id", 4, unsafe.Pointer(&mat)},
	}
	for _, r := range reads {
		if err := g.read(r.name, i, r.size, r.dst); err != nil {
			return Fragment{}, err
		}
	}
	f.Ok = f.TriID != 0xFFFFFFFF // PR_TRI_NONE
	f.X, f.Y = x, y
	f.U, f.V, f.Du, f.Dv = uvd[0], uvd[1], uvd[2], uvd[3]
	f.MaterialID = int64(mat)
	return f, nil
}

// Image reads the frame's RGBA8 image (the buffer.Image() layout).
func (g *GBuffer) Image() (*image.RGBA, error) {
	img := image.NewRGBA(image.Rect(0, 0, g.W, g.H))
	err := check(prDeviceRead(g.dev.ctx, g.fields["rgba"], uintptr(len(img.Pix)), unsafe.Pointer(&img.Pix[0])))
	return img, err
}

// Free releases the device memory.
func (g *GBuffer) Free() error {
	var err error
	for name, p := range g.fields {
		if p != nil {
			if e := check(prDeviceFree(g.dev.ctx, p)); e != nil && err == nil {
				err = e
			}
		}
		delete(g.fields, name)
	}
	return err
}
