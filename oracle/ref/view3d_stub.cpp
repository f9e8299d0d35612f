// Non-graphics stand-in for MolTwister's C3DView, used only to link the reference CPU MD path
// into the oracle harness.  TEST INFRASTRUCTURE: never linked into the product library.
//
// The MD path touches C3DView only through the box: CMDFFMatrices::CCellList::init and the
// CSimulationBox constructor call the static C3DView::calcPBC() (3DView/MolTwister3DView.cpp:218-271),
// which returns the user-defined periodic box when one is enabled, else the bounding box of the
// atoms of the current frame.  This file defines the members that the MD sources reference, with
// that behaviour; there is no OpenGL/GLUT here and the viewer itself is not reproduced.
#include "3DView/MolTwister3DView.h"
#include <cfloat>

bool C3DView::headless_ = true;
int C3DView::updateRequested_ = 0;
int C3DView::fullscreenRequested_ = 0;
bool C3DView::requestQuit_ = false;
bool C3DView::orthoView_ = false;
bool C3DView::viewAxes_ = false;
bool C3DView::viewIsoSurface_ = false;
bool C3DView::viewBondsAcrossPBC_ = true;
std::vector<std::shared_ptr<CAtom>>* C3DView::atoms_ = nullptr;
std::vector<std::shared_ptr<CGLObject>>* C3DView::glObjects_ = nullptr;
int* C3DView::currentFrame_ = nullptr;
C3DView::CCamera C3DView::camera_;
bool C3DView::leftMButtonPressed_ = false;
bool C3DView::middleMButtonPressed_ = false;
bool C3DView::rightMButtonPressed_ = false;
C3DView::CScreenCoord C3DView::coordLastClick_;
C3DView::CScreenCoord C3DView::lastWindowSize_;
C3DView::CResolution C3DView::primitiveRes_;
C3DView::CArg C3DView::progArg_;
std::vector<C3DVector> C3DView::selColorRot_;
CDefaultAtomicProperties* C3DView::defaultAtProp_ = nullptr;
CExpLookup C3DView::expLookup_;
bool C3DView::applyUserDefPBC_ = false;
C3DRect C3DView::pbcUser_;
C3DRect C3DView::pbc_;
int C3DView::numAtomsBeforeNoDraw_ = 0;
bool C3DView::fogEnabled_ = false;
bool C3DView::labelsVisible_ = false;
int C3DView::labelsFontSize_ = 12;
C3DVector C3DView::backgroundColor_;
bool C3DView::useVanDerWaalsRadiusForAtoms_ = false;
double C3DView::vdwScaleFactor_ = 1.0;

C3DView::CArg::~CArg() {}

C3DView::C3DView(int, char*[]) {}

void C3DView::serialize(CSerializer&, bool, std::vector<std::shared_ptr<CAtom>>* atoms,
                        std::vector<std::shared_ptr<CGLObject>>* glObjects, int* currentFrame,
                        CDefaultAtomicProperties* defAtProp)
{
    if(atoms) atoms_ = atoms;
    if(glObjects) glObjects_ = glObjects;
    if(currentFrame) currentFrame_ = currentFrame;
    if(defAtProp) defaultAtProp_ = defAtProp;
}

C3DVector C3DView::currFrmAtVec(const CAtom& atom)
{
    int frame = currentFrame_ ? *currentFrame_ : 0;
    if(frame < 0 || frame >= (int)atom.r_.size()) return C3DVector();
    return atom.r_[(size_t)frame];
}

// Box used by the MD engine: the user PBC when enabled, else the atoms' bounding box, with
// degenerate (<1e-5) widths padded by +-1 (same rule as the viewer's calcPBC).
C3DRect C3DView::calcPBC(int frame)
{
    C3DRect box;
    if(applyUserDefPBC_)
    {
        box = pbcUser_;
    }
    else if(atoms_ && !atoms_->empty())
    {
        const double big = static_cast<double>(FLT_MAX);
        box.rLow_ = C3DVector(big, big, big);
        box.rHigh_ = C3DVector(-big, -big, -big);
        for(const auto& a : *atoms_)
        {
            C3DVector r;
            if(currentFrame_ && frame < 0) r = currFrmAtVec(*a);
            else if(frame >= 0 && frame < (int)a->r_.size()) r = a->r_[(size_t)frame];
            else return C3DRect(C3DVector(-1.0, -1.0, -1.0), C3DVector(1.0, 1.0, 1.0));
            if(r.x_ < box.rLow_.x_) box.rLow_.x_ = r.x_;
            if(r.y_ < box.rLow_.y_) box.rLow_.y_ = r.y_;
            if(r.z_ < box.rLow_.z_) box.rLow_.z_ = r.z_;
            if(r.x_ > box.rHigh_.x_) box.rHigh_.x_ = r.x_;
            if(r.y_ > box.rHigh_.y_) box.rHigh_.y_ = r.y_;
            if(r.z_ > box.rHigh_.z_) box.rHigh_.z_ = r.z_;
        }
    }
    else
    {
        box = C3DRect(C3DVector(-1.0, -1.0, -1.0), C3DVector(1.0, 1.0, 1.0));
    }
    if(box.getWidthX() < 1E-5) { box.rLow_.x_ -= 1.0; box.rHigh_.x_ += 1.0; }
    if(box.getWidthY() < 1E-5) { box.rLow_.y_ -= 1.0; box.rHigh_.y_ += 1.0; }
    if(box.getWidthZ() < 1E-5) { box.rLow_.z_ -= 1.0; box.rHigh_.z_ += 1.0; }
    return box;
}
