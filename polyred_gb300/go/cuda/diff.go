package cuda

// Differentiable deferred shading for Go hosts: a Forward/Backward pair over
// pr_diff_forward / pr_diff_backward (include/polyred_cuda.h, section
// "differentiable deferred shading"). It keeps the contract of
// torch.autograd.Function that the Python host follows
// (polyred_gb300/diff.py, ShadeFunction): Forward computes the output and
// saves what Backward needs (here the differentiation G-buffer, the frame and
// the parameters it was given); Backward takes dL/d(output) and returns a
// gradient for each input that asked for one (a nil pointer in DiffGrads is
// an input that needs none), recomputing every interpolated attribute and
// per-light term from the saved G-buffer instead of storing them. Visibility
// (triangle IDs, shadow and AO factors) is held fixed by that G-buffer.
//
// The reference has no gradients; the forward frame is its Render()
// (render/raster.go:155-199) up to the pre-Round radiance of FragmentShader
// (shader/blinn_cpu.go:24-106).

import (
	"runtime"
	"unsafe"
)

// DGBFloats is the differentiation G-buffer's floats per pixel (PR_DGB_FLOATS).
const DGBFloats = 16

// DiffParams mirrors pr_diff_params: the differentiable parameters. Vertex
// arrays are device memory ([n_tris][3][4] float32, e.g. from DeviceAlloc);
// material arrays are host memory. A nil field keeps the scene's value.
type DiffParams struct {
	Size         uint32
	NMaterials   uint32
	VertexColor  unsafe.Pointer // DEVICE [n_tris][3][4], RGBA in [0, 1]
	VertexNormal unsafe.Pointer // DEVICE [n_tris][3][4], object space
	Kd           *float32       // HOST [n_materials][3], Diffuse/255
	Ks           *float32       // HOST [n_materials][3], Specular/255
	Shininess    *float32       // HOST [n_materials]
}

// DiffGrads mirrors pr_diff_grads: where Backward writes each gradient. The
// vertex gradients are device memory, the others host memory; nil: not wanted.
type DiffGrads struct {
	Size           uint32
	_              uint32
	VertexColor    unsafe.Pointer // DEVICE [n_tris][3][4], overwritten
	VertexNormal   unsafe.Pointer // DEVICE [n_tris][3][4] (w = 0), overwritten
	Kd             *float64       // HOST [n_materials][3]
	Ks             *float64       // HOST [n_materials][3]
	Shininess      *float64       // HOST [n_materials]
	LightPos       *float64       // HOST [n_lights][3] (0 for directional lights)
	LightIntensity *float64       // HOST [n_lights]
	Ambient        *float64       // HOST [n_ambient]
}

var (
	prDiffForward  func(ctx uintptr, f *FrameDesc, p *DiffParams, radiance, gbuf unsafe.Pointer, o *Outputs) int32
	prDiffBackward func(ctx uintptr, f *FrameDesc, p *DiffParams, gbuf, grad unsafe.Pointer, g *DiffGrads) int32
)

func init() {
	registerExtra = append(registerExtra, func(lib uintptr) error {
		if err := register(&prDiffForward, lib, "pr_diff_forward"); err != nil {
			return err
		}
		return register(&prDiffBackward, lib, "pr_diff_backward")
	})
}

// Shade is one differentiable view of the device's scene: a Forward/Backward
// pair with device buffers for the radiance ([H][W][4] float32) and the
// differentiation G-buffer ([H][W][DGBFloats] float32), rows top-down.
type Shade struct {
	dev      *Device
	W, H     int
	Radiance unsafe.Pointer // DEVICE, written by Forward
	gbuf     unsafe.Pointer
	frame    FrameDesc
	params   DiffParams
	saved    bool
}

// NewShade allocates the radiance and G-buffer of w x h frames on d.
func (d *Device) NewShade(w, h int) (*Shade, error) {
	if w <= 0 || h <= 0 {
		return nil, &Error{Status: ErrInvalidArg, Detail: "Shade size must be positive"}
	}
	d.mu.Lock()
	ctx := d.ctx
	d.mu.Unlock()
	if ctx == 0 {
		return nil, ErrClosed
	}
	s := &Shade{dev: d, W: w, H: h}
	if err := check(prDeviceAlloc(ctx, uintptr(w*h*4*4), &s.Radiance)); err != nil {
		return nil, err
	}
	if err := check(prDeviceAlloc(ctx, uintptr(w*h*DGBFloats*4), &s.gbuf)); err != nil {
		s.Free()
		return nil, err
	}
	runtime.SetFinalizer(s, func(s *Shade) { s.Free() })
	return s, nil
}

// Forward renders frame f (size W x H) as the first Render() of a new
// renderer (the shadow maps start zeroed) with parameters p, writes the float
// radiance to s.Radiance and saves the G-buffer, f and p for Backward.
func (s *Shade) Forward(f *FrameDesc, p *DiffParams) error {
	d := s.dev
	d.mu.Lock()
	defer d.mu.Unlock()
	if d.ctx == 0 || s.gbuf == nil {
		return ErrClosed
	}
	if int(f.Width) != s.W || int(f.Height) != s.H {
		return &Error{Status: ErrInvalidArg, Detail: "frame size differs from the Shade's"}
	}
	f.Size = uint32(unsafe.Sizeof(*f))
	p.Size = uint32(unsafe.Sizeof(*p))
	s.saved = false
	if err := check(prShadowReset(d.ctx)); err != nil {
		return err
	}
	if err := check(prDiffForward(d.ctx, f, p, s.Radiance, s.gbuf, nil)); err != nil {
		return err
	}
	s.frame, s.params, s.saved = *f, *p, true
	runtime.KeepAlive(f)
	runtime.KeepAlive(p)
	return nil
}

// Backward takes dL/d(radiance) (DEVICE [H][W][4] float32, alpha ignored) and
// writes the gradients g asks for, for the frame and parameters of the last
// Forward. The parameter arrays given to Forward must be unchanged.
func (s *Shade) Backward(gradRadiance unsafe.Pointer, g *DiffGrads) error {
	d := s.dev
	d.mu.Lock()
	defer d.mu.Unlock()
	if d.ctx == 0 || s.gbuf == nil {
		return ErrClosed
	}
	if !s.saved {
		return &Error{Status: ErrInvalidArg, Detail: "Backward before Forward"}
	}
	g.Size = uint32(unsafe.Sizeof(*g))
	err := check(prDiffBackward(d.ctx, &s.frame, &s.params, s.gbuf, gradRadiance, g))
	runtime.KeepAlive(g)
	return err
}

// ReadRadiance copies the radiance of the last Forward into dst
// (len(dst) >= W*H*4).
func (s *Shade) ReadRadiance(dst []float32) error {
	if len(dst) < s.W*s.H*4 {
		return &Error{Status: ErrInvalidArg, Detail: "ReadRadiance: destination too small"}
	}
	return check(prDeviceRead(s.dev.ctx, s.Radiance, uintptr(s.W*s.H*16), unsafe.Pointer(&dst[0])))
}

// Free releases the device buffers.
func (s *Shade) Free() error {
	var err error
	for _, p := range []*unsafe.Pointer{&s.Radiance, &s.gbuf} {
		if *p != nil {
			if e := check(prDeviceFree(s.dev.ctx, *p)); e != nil && err == nil {
				err = e
			}
			*p = nil
		}
	}
	s.saved = false
	return err
}
